// gs_rasterizer.cu -- differentiable Gaussian-splatting tile rasterizer for
// sm_103a (the renderer the simulated particles feed in end-to-end mode).
//
// Frame = preprocess (one thread per Gaussian: view transform, EWA 2D
// covariance with the 0.3 px low-pass, conic, 3-sigma radius, tile rect,
// SH color, normal) -> prefix sum of tiles touched -> one (tile|depth, id)
// pair per touched tile -> stable CUB radix sort -> tile ranges -> render
// (one 16x16 block per tile, batches of 256 Gaussians staged in shared
// memory, front-to-back blending with alpha = min(0.99, o e^power), pairs
// with alpha < 1/255 skipped, a pixel stops before its transmittance would
// fall below 1e-4).  Semantics follow rasterizer_impl.cu:54-116 and
// forward.cu:204-455 of the reference's diff_gauss rasterizer.
//
// The backward is the exact derivative of that forward (so a clamped alpha
// = 0.99 passes no gradient) and reduces each Gaussian's per-pixel terms
// across the warp before one atomic per warp: every lane of a block walks
// the same tile list in the same order, so at each step the warp works on
// one Gaussian.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <cmath>
#include <cstdint>
#include <type_traits>

#include "../../include/gsplat.h"
#include "../../include/mpm.h"
#include "mpm_launch.h"

namespace mpm {
namespace {

constexpr int kT = GS_TILE;
constexpr int kBlock = kT * kT;

// real spherical-harmonics normalisation constants, degrees 0-3
constexpr float kY0 = 0.28209479177387814f;
constexpr float kY1 = 0.4886025119029199f;
__constant__ float kY2[5] = {1.0925484305920792f, -1.0925484305920792f, 0.31539156525252005f, -1.0925484305920792f,
                          0.5462742152960396f};
__constant__ float kY3[7] = {-0.5900435899266435f, 2.890611442640554f, -0.4570457994644658f, 0.3731763325901154f,
                          -0.4570457994644658f, 1.445305721320277f, -0.5900435899266435f};

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return {x, y, z}; }

// rasterizer matrix convention: x' = m[0]x + m[4]y + m[8]z + m[12]
__device__ __forceinline__ V3 xform43(const float* m, V3 p)
{
    return v3(m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12], m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13],
              m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14]);
}
__device__ __forceinline__ float xform44w(const float* m, V3 p)
{
    return m[3] * p.x + m[7] * p.y + m[11] * p.z + m[15];
}

// pixel coordinate of an NDC coordinate (evaluated in double as the reference does)
__device__ __forceinline__ float ndc_to_pix(float v, int S) { return (float)((((double)v + 1.0) * S - 1.0) * 0.5); }

// rotation matrix of the quaternion (r,x,y,z) as given (row-major)
__device__ __forceinline__ void quat_rot(const float* q, float* R)
{
    const float r = q[0], x = q[1], y = q[2], z = q[3];
    R[0] = 1.f - 2.f * (y * y + z * z);
    R[1] = 2.f * (x * y - r * z);
    R[2] = 2.f * (x * z + r * y);
    R[3] = 2.f * (x * y + r * z);
    R[4] = 1.f - 2.f * (x * x + z * z);
    R[5] = 2.f * (y * z - r * x);
    R[6] = 2.f * (x * z - r * y);
    R[7] = 2.f * (y * z + r * x);
    R[8] = 1.f - 2.f * (x * x + y * y);
}

// normal axis of a Gaussian: the local axis of smallest scale (ties as the
// reference's branch order), as a column of R
__device__ __forceinline__ int normal_axis(const float* s)
{
    if (s[0] > s[2] && s[1] > s[2]) return 2;
    if (s[0] > s[1] && s[2] > s[1]) return 1;
    return 0;
}

// SH basis values at unit direction d, degree <= 3
__device__ __forceinline__ void sh_basis(int deg, V3 d, float* b)
{
    const float x = d.x, y = d.y, z = d.z;
    b[0] = kY0;
    if (deg < 1) return;
    b[1] = -kY1 * y;
    b[2] = kY1 * z;
    b[3] = -kY1 * x;
    if (deg < 2) return;
    const float xx = x * x, yy = y * y, zz = z * z;
    b[4] = kY2[0] * x * y;
    b[5] = kY2[1] * y * z;
    b[6] = kY2[2] * (2.f * zz - xx - yy);
    b[7] = kY2[3] * x * z;
    b[8] = kY2[4] * (xx - yy);
    if (deg < 3) return;
    b[9] = kY3[0] * y * (3.f * xx - yy);
    b[10] = kY3[1] * x * y * z;
    b[11] = kY3[2] * y * (4.f * zz - xx - yy);
    b[12] = kY3[3] * z * (2.f * zz - 3.f * xx - 3.f * yy);
    b[13] = kY3[4] * x * (4.f * zz - xx - yy);
    b[14] = kY3[5] * z * (xx - yy);
    b[15] = kY3[6] * x * (xx - 3.f * yy);
}

// d b_k / d(x,y,z) for k >= 1
__device__ __forceinline__ void sh_basis_grad(int deg, V3 d, float (*g)[3])
{
    const float x = d.x, y = d.y, z = d.z;
    for (int k = 0; k < 16; ++k) g[k][0] = g[k][1] = g[k][2] = 0.f;
    if (deg < 1) return;
    g[1][1] = -kY1;
    g[2][2] = kY1;
    g[3][0] = -kY1;
    if (deg < 2) return;
    const float xx = x * x, yy = y * y, zz = z * z;
    g[4][0] = kY2[0] * y, g[4][1] = kY2[0] * x;
    g[5][1] = kY2[1] * z, g[5][2] = kY2[1] * y;
    g[6][0] = -2.f * kY2[2] * x, g[6][1] = -2.f * kY2[2] * y, g[6][2] = 4.f * kY2[2] * z;
    g[7][0] = kY2[3] * z, g[7][2] = kY2[3] * x;
    g[8][0] = 2.f * kY2[4] * x, g[8][1] = -2.f * kY2[4] * y;
    if (deg < 3) return;
    g[9][0] = kY3[0] * 6.f * x * y, g[9][1] = kY3[0] * (3.f * xx - 3.f * yy);
    g[10][0] = kY3[1] * y * z, g[10][1] = kY3[1] * x * z, g[10][2] = kY3[1] * x * y;
    g[11][0] = -2.f * kY3[2] * x * y, g[11][1] = kY3[2] * (4.f * zz - xx - 3.f * yy), g[11][2] = 8.f * kY3[2] * y * z;
    g[12][0] = -6.f * kY3[3] * x * z, g[12][1] = -6.f * kY3[3] * y * z,
    g[12][2] = kY3[3] * (6.f * zz - 3.f * xx - 3.f * yy);
    g[13][0] = kY3[4] * (4.f * zz - 3.f * xx - yy), g[13][1] = -2.f * kY3[4] * x * y, g[13][2] = 8.f * kY3[4] * x * z;
    g[14][0] = 2.f * kY3[5] * x * z, g[14][1] = -2.f * kY3[5] * y * z, g[14][2] = kY3[5] * (xx - yy);
    g[15][0] = kY3[6] * (3.f * xx - 3.f * yy), g[15][1] = -6.f * kY3[6] * x * y;
}

struct Frame {
    int P, H, W, gx, gy;
    float fx, fy, limx, limy, mod;
    int deg, M, ED;
};

Frame make_frame(const GsScene& s)
{
    Frame f;
    f.P = s.P;
    f.H = s.H;
    f.W = s.W;
    f.gx = (s.W + kT - 1) / kT;
    f.gy = (s.H + kT - 1) / kT;
    f.fx = s.W / (2.f * s.tanfovx);
    f.fy = s.H / (2.f * s.tanfovy);
    f.limx = 1.3f * s.tanfovx;
    f.limy = 1.3f * s.tanfovy;
    f.mod = s.scale_modifier;
    f.deg = s.sh_degree;
    f.M = s.sh_coeffs;
    f.ED = s.extra_dims;
    return f;
}

// view-space mean with x, y clamped to 1.3 x the field of view (EWA Jacobian point)
struct ViewPt {
    V3 t;            // view-space mean
    float tx, ty;    // clamped x, y
    bool cx, cy;     // clamped?
    float sx, sy;    // sign of the clamp
};

__device__ __forceinline__ ViewPt view_point(const Frame& f, const float* vm, V3 m)
{
    ViewPt v;
    v.t = xform43(vm, m);
    const float txtz = v.t.x / v.t.z, tytz = v.t.y / v.t.z;
    v.cx = txtz < -f.limx || txtz > f.limx;
    v.cy = tytz < -f.limy || tytz > f.limy;
    v.sx = txtz < 0.f ? -1.f : 1.f;
    v.sy = tytz < 0.f ? -1.f : 1.f;
    v.tx = fminf(f.limx, fmaxf(-f.limx, txtz)) * v.t.z;
    v.ty = fminf(f.limy, fmaxf(-f.limy, tytz)) * v.t.z;
    return v;
}

// U = J R_view (2x3), J the EWA Jacobian at the clamped view point
__device__ __forceinline__ void ewa_u(const Frame& f, const float* vm, const ViewPt& v, float* U)
{
    const float iz = 1.f / v.t.z, iz2 = iz * iz;
    const float j00 = f.fx * iz, j02 = -f.fx * v.tx * iz2, j11 = f.fy * iz, j12 = -f.fy * v.ty * iz2;
    // R_view rows: (m0 m4 m8), (m1 m5 m9), (m2 m6 m10)
    U[0] = j00 * vm[0] + j02 * vm[2];
    U[1] = j00 * vm[4] + j02 * vm[6];
    U[2] = j00 * vm[8] + j02 * vm[10];
    U[3] = j11 * vm[1] + j12 * vm[2];
    U[4] = j11 * vm[5] + j12 * vm[6];
    U[5] = j11 * vm[9] + j12 * vm[10];
}

__device__ __forceinline__ void cov3_full(const float* c6, float* S)
{
    S[0] = c6[0], S[1] = c6[1], S[2] = c6[2];
    S[3] = c6[1], S[4] = c6[3], S[5] = c6[4];
    S[6] = c6[2], S[7] = c6[4], S[8] = c6[5];
}

// ------------------------------------------------------------ preprocess

__global__ void k_gs_preprocess(Frame f, GsScene s, GsGeom g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.P) return;
    g.radii[i] = 0;
    g.tiles_touched[i] = 0;
    const V3 m = v3(s.means3D[3 * i], s.means3D[3 * i + 1], s.means3D[3 * i + 2]);
    const ViewPt vp = view_point(f, s.viewmatrix, m);
    if (!(vp.t.z > 0.2f)) return;  // near culling (NaN included)
    const V3 ph = xform43(s.projmatrix, m);
    const float pw = 1.f / (xform44w(s.projmatrix, m) + 0.0000001f);
    const float ppx = ph.x * pw, ppy = ph.y * pw;
    float c6[6];
    if (s.cov3D) {
        for (int k = 0; k < 6; ++k) c6[k] = s.cov3D[6 * i + k];
    } else {
        float R[9], Mx[9];
        quat_rot(s.rotations + 4 * i, R);
        // M = S R^T: glm::mat3's constructor takes the quaternion matrix's
        // rows as columns (forward.cu:134-140), so the reference's Sigma is
        // R S^2 R^T with R as quat_rot writes it
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) Mx[3 * r + c] = f.mod * s.scales[3 * i + r] * R[3 * c + r];
        // Sigma = M^T M
        c6[0] = Mx[0] * Mx[0] + Mx[3] * Mx[3] + Mx[6] * Mx[6];
        c6[1] = Mx[0] * Mx[1] + Mx[3] * Mx[4] + Mx[6] * Mx[7];
        c6[2] = Mx[0] * Mx[2] + Mx[3] * Mx[5] + Mx[6] * Mx[8];
        c6[3] = Mx[1] * Mx[1] + Mx[4] * Mx[4] + Mx[7] * Mx[7];
        c6[4] = Mx[1] * Mx[2] + Mx[4] * Mx[5] + Mx[7] * Mx[8];
        c6[5] = Mx[2] * Mx[2] + Mx[5] * Mx[5] + Mx[8] * Mx[8];
    }
    for (int k = 0; k < 6; ++k) g.cov3D[6 * i + k] = c6[k];
    V3 nrm;
    if (s.norm3D) {
        nrm = v3(s.norm3D[3 * i], s.norm3D[3 * i + 1], s.norm3D[3 * i + 2]);
    } else {
        float R[9];
        quat_rot(s.rotations + 4 * i, R);
        const int a = normal_axis(s.scales + 3 * i);
        // column a of R (transpose(R_glm) * e_a, forward.cu:188)
        nrm = v3(R[a], R[3 + a], R[6 + a]);
        const V3 ray = v3(m.x - s.campos[0], m.y - s.campos[1], m.z - s.campos[2]);
        if (ray.x * nrm.x + ray.y * nrm.y + ray.z * nrm.z > 0.f) nrm = v3(-nrm.x, -nrm.y, -nrm.z);
    }
    // 2D covariance U Sigma U^T + 0.3 I
    float U[6], S[9];
    ewa_u(f, s.viewmatrix, vp, U);
    cov3_full(c6, S);
    float US[6];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 3; ++c)
            US[3 * r + c] = U[3 * r] * S[c] + U[3 * r + 1] * S[3 + c] + U[3 * r + 2] * S[6 + c];
    const float a = US[0] * U[0] + US[1] * U[1] + US[2] * U[2] + 0.3f;
    const float b = US[0] * U[3] + US[1] * U[4] + US[2] * U[5];
    const float c = US[3] * U[3] + US[4] * U[4] + US[5] * U[5] + 0.3f;
    const float det = a * c - b * b;
    if (det == 0.f) return;
    const float idet = 1.f / det;
    const float mid = 0.5f * (a + c);
    const float l1 = mid + sqrtf(fmaxf(0.1f, mid * mid - det)), l2 = mid - sqrtf(fmaxf(0.1f, mid * mid - det));
    const float rad = ceilf(3.f * sqrtf(fmaxf(l1, l2)));
    const float px = ndc_to_pix(ppx, f.W), py = ndc_to_pix(ppy, f.H);
    const int r = (int)rad;
    const int x0 = min(f.gx, max(0, (int)((px - r) / kT))), y0 = min(f.gy, max(0, (int)((py - r) / kT)));
    const int x1 = min(f.gx, max(0, (int)((px + r + kT - 1) / kT))), y1 = min(f.gy, max(0, (int)((py + r + kT - 1) / kT)));
    if ((x1 - x0) * (y1 - y0) == 0) return;
    float rgb[3];
    if (s.colors) {
        for (int k = 0; k < 3; ++k) rgb[k] = s.colors[3 * i + k];
        g.clamped[3 * i] = g.clamped[3 * i + 1] = g.clamped[3 * i + 2] = 0;
    } else {
        V3 d = v3(m.x - s.campos[0], m.y - s.campos[1], m.z - s.campos[2]);
        const float il = 1.f / sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
        d = v3(d.x * il, d.y * il, d.z * il);
        float bs[16];
        sh_basis(f.deg, d, bs);
        const int nb = (f.deg + 1) * (f.deg + 1);
        for (int ch = 0; ch < 3; ++ch) {
            float v = 0.f;
            for (int k = 0; k < nb; ++k) v += bs[k] * s.shs[((long long)i * f.M + k) * 3 + ch];
            v += 0.5f;
            g.clamped[3 * i + ch] = v < 0.f;
            rgb[ch] = fmaxf(v, 0.f);
        }
    }
    for (int k = 0; k < 3; ++k) g.rgb[3 * i + k] = rgb[k];
    g.normal[3 * i] = nrm.x, g.normal[3 * i + 1] = nrm.y, g.normal[3 * i + 2] = nrm.z;
    g.depth[i] = vp.t.z;
    g.radii[i] = r;
    g.xy[2 * i] = px, g.xy[2 * i + 1] = py;
    g.conic_opacity[4 * i] = c * idet;
    g.conic_opacity[4 * i + 1] = -b * idet;
    g.conic_opacity[4 * i + 2] = a * idet;
    g.conic_opacity[4 * i + 3] = s.opacities[i];
    g.tiles_touched[i] = (uint32_t)((x1 - x0) * (y1 - y0));
}

// ------------------------------------------------------------ binning

__global__ void k_gs_duplicate(Frame f, GsGeom g, uint64_t* keys, uint32_t* ids)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.P || g.radii[i] <= 0) return;
    uint32_t off = i == 0 ? 0 : g.offsets[i - 1];
    const float px = g.xy[2 * i], py = g.xy[2 * i + 1];
    const int r = g.radii[i];
    const int x0 = min(f.gx, max(0, (int)((px - r) / kT))), y0 = min(f.gy, max(0, (int)((py - r) / kT)));
    const int x1 = min(f.gx, max(0, (int)((px + r + kT - 1) / kT))), y1 = min(f.gy, max(0, (int)((py + r + kT - 1) / kT)));
    const uint32_t dbits = __float_as_uint(g.depth[i]);  // depth > 0.2: the bits order like the values
    for (int y = y0; y < y1; ++y)
        for (int x = x0; x < x1; ++x) {
            keys[off] = ((uint64_t)(y * f.gx + x) << 32) | dbits;
            ids[off] = (uint32_t)i;
            ++off;
        }
}

__global__ void k_gs_ranges(int L, const uint64_t* keys, uint32_t* ranges)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L) return;
    const uint32_t t = (uint32_t)(keys[i] >> 32);
    if (i == 0 || (uint32_t)(keys[i - 1] >> 32) != t) ranges[2 * t] = i;
    if (i == L - 1 || (uint32_t)(keys[i + 1] >> 32) != t) ranges[2 * t + 1] = i + 1;
}

// ------------------------------------------------------------ render

template <int EDMAX>
__global__ void __launch_bounds__(kBlock) k_gs_render(Frame f, GsScene s, GsGeom g, const uint32_t* ids,
                                                      const uint32_t* ranges, GsImage img)
{
    __shared__ int sid[kBlock];
    __shared__ float2 sxy[kBlock];
    __shared__ float4 sco[kBlock];
    const int tile = blockIdx.y * f.gx + blockIdx.x;
    const int tr = threadIdx.y * kT + threadIdx.x;
    const int px = blockIdx.x * kT + threadIdx.x, py = blockIdx.y * kT + threadIdx.y;
    const bool inside = px < f.W && py < f.H;
    const float pfx = (float)px, pfy = (float)py;
    const uint32_t r0 = ranges[2 * tile], r1 = ranges[2 * tile + 1];
    const int n = (int)(r1 - r0);
    bool done = !inside;
    float T = 1.f, C[3] = {0.f, 0.f, 0.f}, D = 0.f, N[3] = {0.f, 0.f, 0.f}, E[EDMAX > 0 ? EDMAX : 1];
#pragma unroll
    for (int e = 0; e < (EDMAX > 0 ? EDMAX : 1); ++e) E[e] = 0.f;
    uint32_t contributor = 0, last = 0;
    for (int base = 0; base < n; base += kBlock) {
        if (__syncthreads_count(done) == kBlock) break;
        if (base + tr < n) {
            const int id = (int)ids[r0 + base + tr];
            sid[tr] = id;
            sxy[tr] = make_float2(g.xy[2 * id], g.xy[2 * id + 1]);
            sco[tr] = reinterpret_cast<const float4*>(g.conic_opacity)[id];
        }
        __syncthreads();
        const int cnt = min(kBlock, n - base);
        for (int j = 0; !done && j < cnt; ++j) {
            ++contributor;
            const float dx = sxy[j].x - pfx, dy = sxy[j].y - pfy;
            const float4 co = sco[j];
            const float power = -0.5f * (co.x * dx * dx + co.z * dy * dy) - co.y * dx * dy;
            if (power > 0.f) continue;
            const float alpha = fminf(0.99f, co.w * expf(power));
            if (alpha < 1.f / 255.f) continue;
            const float nT = T * (1.f - alpha);
            if (nT < 0.0001f) {
                done = true;
                continue;
            }
            const int id = sid[j];
            const float w = alpha * T;
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                C[ch] += g.rgb[3 * id + ch] * w;
                N[ch] += g.normal[3 * id + ch] * w;
            }
            D += g.depth[id] * w;
#pragma unroll
            for (int e = 0; e < EDMAX; ++e)
                if (e < f.ED) E[e] += s.extra[(long long)id * f.ED + e] * w;
            T = nT;
            last = contributor;
        }
    }
    if (!inside) return;
    const long long pix = (long long)py * f.W + px, HW = (long long)f.H * f.W;
    img.alpha[pix] = 1.f - T;
    img.n_contrib[pix] = last;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        img.color[ch * HW + pix] = C[ch] + T * s.bg[ch];
        img.normal[ch * HW + pix] = N[ch];
    }
    img.depth[pix] = D;
#pragma unroll
    for (int e = 0; e < EDMAX; ++e)
        if (e < f.ED) img.extra[e * HW + pix] = E[e];
}

// ------------------------------------------------------------ backward

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// adjoint of k_gs_render: per pixel, walk the tile list back to front,
// recovering T by division; the per-Gaussian terms are summed over the warp.
// HD / HN: the depth / normal images have a gradient (otherwise their terms
// vanish and are not formed)
template <int EDMAX, bool HD, bool HN>
__global__ void __launch_bounds__(kBlock) k_gs_render_bwd(Frame f, GsScene s, GsGeom g, const uint32_t* ids,
                                                          const uint32_t* ranges, GsImage img, const float* dLc,
                                                          const float* dLd, const float* dLn, const float* dLa,
                                                          const float* dLe, GsGrads gr)
{
    __shared__ int sid[kBlock];
    __shared__ float2 sxy[kBlock];
    __shared__ float4 sco[kBlock];
    const int tile = blockIdx.y * f.gx + blockIdx.x;
    const int tr = threadIdx.y * kT + threadIdx.x;
    const int lane = tr & 31;
    const int px = blockIdx.x * kT + threadIdx.x, py = blockIdx.y * kT + threadIdx.y;
    const bool inside = px < f.W && py < f.H;
    const float pfx = (float)px, pfy = (float)py;
    const uint32_t r0 = ranges[2 * tile], r1 = ranges[2 * tile + 1];
    const int n = (int)(r1 - r0);
    const long long pix = inside ? (long long)py * f.W + px : 0, HW = (long long)f.H * f.W;
    const float Tf = inside ? 1.f - img.alpha[pix] : 0.f;
    const int last = inside ? (int)img.n_contrib[pix] : 0;
    float gc[3] = {0.f, 0.f, 0.f}, gn[3] = {0.f, 0.f, 0.f}, gd = 0.f, ga = 0.f, ge[EDMAX > 0 ? EDMAX : 1];
    if (inside) {
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            gc[ch] = dLc ? dLc[ch * HW + pix] : 0.f;
            gn[ch] = dLn ? dLn[ch * HW + pix] : 0.f;
        }
        gd = dLd ? dLd[pix] : 0.f;
        ga = dLa ? dLa[pix] : 0.f;
    }
#pragma unroll
    for (int e = 0; e < (EDMAX > 0 ? EDMAX : 1); ++e) ge[e] = (inside && dLe && e < f.ED) ? dLe[e * HW + pix] : 0.f;
    const float bg_dot = gc[0] * s.bg[0] + gc[1] * s.bg[1] + gc[2] * s.bg[2];
    float T = Tf;
    // blended value of everything behind the current Gaussian (normalised)
    float acc_c[3] = {0.f, 0.f, 0.f}, acc_n[3] = {0.f, 0.f, 0.f}, acc_d = 0.f, acc_e[EDMAX > 0 ? EDMAX : 1];
    float prev_a = 0.f, prev_c[3] = {0.f, 0.f, 0.f}, prev_n[3] = {0.f, 0.f, 0.f}, prev_d = 0.f,
          prev_e[EDMAX > 0 ? EDMAX : 1];
#pragma unroll
    for (int e = 0; e < (EDMAX > 0 ? EDMAX : 1); ++e) acc_e[e] = prev_e[e] = 0.f;
    const float hx = 0.5f * f.W, hy = 0.5f * f.H;
    // no pixel of the tile blends anything past the largest last contributor:
    // start the walk there instead of at the end of the tile list
    __shared__ int s_top;
    if (tr == 0) s_top = 0;
    __syncthreads();
    const int wmax = __reduce_max_sync(0xffffffffu, last);
    if (lane == 0) atomicMax(&s_top, wmax);
    __syncthreads();
    const int ntop = min(s_top, n);
    // walk [0, ntop) backwards in batches; position k (0-based) is contributor k+1
    for (int top = ntop; top > 0; top -= kBlock) {
        __syncthreads();
        const int cnt = min(kBlock, top);
        if (tr < cnt) {
            const int id = (int)ids[r0 + top - 1 - tr];
            sid[tr] = id;
            sxy[tr] = make_float2(g.xy[2 * id], g.xy[2 * id + 1]);
            sco[tr] = reinterpret_cast<const float4*>(g.conic_opacity)[id];
        }
        __syncthreads();
        for (int j = 0; j < cnt; ++j) {
            const int k = top - 1 - j;  // position in the tile list
            const int id = sid[j];
            bool act = inside && k < last;
            float alpha = 0.f, G = 0.f, dx = 0.f, dy = 0.f;
            const float4 co = sco[j];
            if (act) {
                dx = sxy[j].x - pfx;
                dy = sxy[j].y - pfy;
                const float power = -0.5f * (co.x * dx * dx + co.z * dy * dy) - co.y * dx * dy;
                if (power > 0.f) {
                    act = false;
                } else {
                    G = expf(power);
                    alpha = fminf(0.99f, co.w * G);
                    if (alpha < 1.f / 255.f) act = false;
                }
            }
            float o_c[3] = {0.f, 0.f, 0.f}, o_n[3] = {0.f, 0.f, 0.f}, o_d = 0.f, o_o = 0.f, o_x = 0.f, o_y = 0.f,
                  o_a = 0.f, o_b = 0.f, o_cc = 0.f, o_e[EDMAX > 0 ? EDMAX : 1];
#pragma unroll
            for (int e = 0; e < (EDMAX > 0 ? EDMAX : 1); ++e) o_e[e] = 0.f;
            if (act) {
                T = T / (1.f - alpha);
                const float w = alpha * T;
                float dLdalpha = 0.f;
#pragma unroll
                for (int ch = 0; ch < 3; ++ch) {
                    acc_c[ch] = prev_a * prev_c[ch] + (1.f - prev_a) * acc_c[ch];
                    const float c = g.rgb[3 * id + ch];
                    prev_c[ch] = c;
                    dLdalpha += (c - acc_c[ch]) * gc[ch];
                    o_c[ch] = w * gc[ch];
                    if (HN) {
                        acc_n[ch] = prev_a * prev_n[ch] + (1.f - prev_a) * acc_n[ch];
                        const float nn = g.normal[3 * id + ch];
                        prev_n[ch] = nn;
                        dLdalpha += (nn - acc_n[ch]) * gn[ch];
                        o_n[ch] = w * gn[ch];
                    }
                }
                if (HD) {
                    acc_d = prev_a * prev_d + (1.f - prev_a) * acc_d;
                    const float dd = g.depth[id];
                    prev_d = dd;
                    dLdalpha += (dd - acc_d) * gd;
                    o_d = w * gd;
                }
#pragma unroll
                for (int e = 0; e < EDMAX; ++e)
                    if (e < f.ED) {
                        acc_e[e] = prev_a * prev_e[e] + (1.f - prev_a) * acc_e[e];
                        const float ev = s.extra[(long long)id * f.ED + e];
                        prev_e[e] = ev;
                        dLdalpha += (ev - acc_e[e]) * ge[e];
                        o_e[e] = w * ge[e];
                    }
                dLdalpha *= T;
                prev_a = alpha;
                // background and the alpha output: d T_final / d alpha = -T_final / (1 - alpha)
                dLdalpha += (ga - bg_dot) * Tf / (1.f - alpha);
                if (co.w * G < 0.99f) {  // alpha = o G (not clamped)
                    o_o = G * dLdalpha;
                    const float dLdp = dLdalpha * co.w * G;  // d alpha / d power = o G
                    o_x = dLdp * (-co.x * dx - co.y * dy) * hx;
                    o_y = dLdp * (-co.z * dy - co.y * dx) * hy;
                    o_a = dLdp * (-0.5f * dx * dx);
                    o_b = dLdp * (-dx * dy);
                    o_cc = dLdp * (-0.5f * dy * dy);
                }
            }
            if (__any_sync(0xffffffffu, act)) {  // the whole warp works on Gaussian id
                const float r_c0 = warp_sum(o_c[0]), r_c1 = warp_sum(o_c[1]), r_c2 = warp_sum(o_c[2]);
                const float r_n0 = HN ? warp_sum(o_n[0]) : 0.f, r_n1 = HN ? warp_sum(o_n[1]) : 0.f,
                            r_n2 = HN ? warp_sum(o_n[2]) : 0.f;
                const float r_d = HD ? warp_sum(o_d) : 0.f, r_o = warp_sum(o_o), r_x = warp_sum(o_x),
                            r_y = warp_sum(o_y);
                const float r_a = warp_sum(o_a), r_b = warp_sum(o_b), r_cc = warp_sum(o_cc);
                float r_e[EDMAX > 0 ? EDMAX : 1];
#pragma unroll
                for (int e = 0; e < EDMAX; ++e) r_e[e] = warp_sum(o_e[e]);
                if (lane == 0) {
                    atomicAdd(&gr.colors[3 * id], r_c0);
                    atomicAdd(&gr.colors[3 * id + 1], r_c1);
                    atomicAdd(&gr.colors[3 * id + 2], r_c2);
                    if (HN) {
                        atomicAdd(&gr.norm3D[3 * id], r_n0);
                        atomicAdd(&gr.norm3D[3 * id + 1], r_n1);
                        atomicAdd(&gr.norm3D[3 * id + 2], r_n2);
                    }
                    if (HD) atomicAdd(&gr.depth[id], r_d);
                    atomicAdd(&gr.opacities[id], r_o);
                    atomicAdd(&gr.means2D[3 * id], r_x);
                    atomicAdd(&gr.means2D[3 * id + 1], r_y);
                    atomicAdd(&gr.conic[3 * id], r_a);
                    atomicAdd(&gr.conic[3 * id + 1], r_b);
                    atomicAdd(&gr.conic[3 * id + 2], r_cc);
#pragma unroll
                    for (int e = 0; e < EDMAX; ++e)
                        if (e < f.ED && gr.extra) atomicAdd(&gr.extra[(long long)id * f.ED + e], r_e[e]);
                }
            }
        }
    }
}

// adjoint of k_gs_preprocess: conic -> 2D covariance -> 3D covariance and
// view point -> mean; scale/rotation; normal; SH color; projection; depth
__global__ void k_gs_preprocess_bwd(Frame f, GsScene s, GsGeom g, GsGrads gr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.P || g.radii[i] <= 0) return;
    const V3 m = v3(s.means3D[3 * i], s.means3D[3 * i + 1], s.means3D[3 * i + 2]);
    const float* vm = s.viewmatrix;
    const float* pm = s.projmatrix;
    float dm[3] = {0.f, 0.f, 0.f};
    // 1. projection: d(ndc xy)/d mean
    {
        const V3 ph = xform43(pm, m);
        const float iw = 1.f / (xform44w(pm, m) + 0.0000001f);
        const float gx = gr.means2D[3 * i], gy = gr.means2D[3 * i + 1];
        for (int k = 0; k < 3; ++k) {
            const float w3 = pm[4 * k + 3];
            dm[k] += gx * (pm[4 * k] * iw - ph.x * iw * iw * w3) + gy * (pm[4 * k + 1] * iw - ph.y * iw * iw * w3);
        }
    }
    // 2. conic -> 2D covariance (a,b,c)
    const float4 co = reinterpret_cast<const float4*>(g.conic_opacity)[i];
    const float ga = gr.conic[3 * i], gb = gr.conic[3 * i + 1], gc = gr.conic[3 * i + 2];
    // Q = [[A, B],[B, C]], dL/dQ symmetric with off-diagonal gb/2; dL/dSigma2 = -Q dL/dQ Q
    const float qa = co.x, qb = co.y, qc = co.z;
    const float h00 = ga, h01 = 0.5f * gb, h11 = gc;
    const float t00 = qa * h00 + qb * h01, t01 = qa * h01 + qb * h11, t10 = qb * h00 + qc * h01, t11 = qb * h01 + qc * h11;
    const float s00 = -(t00 * qa + t01 * qb), s01 = -(t00 * qb + t01 * qc), s11 = -(t10 * qb + t11 * qc);
    // 3. 2D covariance -> 3D covariance and U = J R_view
    const ViewPt vp = view_point(f, vm, m);
    float U[6], S[9];
    ewa_u(f, vm, vp, U);
    cov3_full(g.cov3D + 6 * i, S);
    const float Gs[4] = {s00, s01, s01, s11};  // dL/dSigma2 (symmetric)
    float dS[9];                                 // U^T G U
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            dS[3 * r + c] = U[r] * (Gs[0] * U[c] + Gs[1] * U[3 + c]) + U[3 + r] * (Gs[2] * U[c] + Gs[3] * U[3 + c]);
    gr.cov3D[6 * i] = dS[0];
    gr.cov3D[6 * i + 1] = dS[1] + dS[3];
    gr.cov3D[6 * i + 2] = dS[2] + dS[6];
    gr.cov3D[6 * i + 3] = dS[4];
    gr.cov3D[6 * i + 4] = dS[5] + dS[7];
    gr.cov3D[6 * i + 5] = dS[8];
    // dL/dU = 2 G U S; dL/dJ = dL/dU R_view^T
    float US[6];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 3; ++c)
            US[3 * r + c] = U[3 * r] * S[c] + U[3 * r + 1] * S[3 + c] + U[3 * r + 2] * S[6 + c];
    float dU[6];
    for (int c = 0; c < 3; ++c) {
        dU[c] = 2.f * (Gs[0] * US[c] + Gs[1] * US[3 + c]);
        dU[3 + c] = 2.f * (Gs[2] * US[c] + Gs[3] * US[3 + c]);
    }
    // R_view rows r_k = (vm[k], vm[4+k], vm[8+k]); U row0 = j00 r_0 + j02 r_2, row1 = j11 r_1 + j12 r_2
    const float dj00 = dU[0] * vm[0] + dU[1] * vm[4] + dU[2] * vm[8];
    const float dj02 = dU[0] * vm[2] + dU[1] * vm[6] + dU[2] * vm[10];
    const float dj11 = dU[3] * vm[1] + dU[4] * vm[5] + dU[5] * vm[9];
    const float dj12 = dU[3] * vm[2] + dU[4] * vm[6] + dU[5] * vm[10];
    const float iz = 1.f / vp.t.z, iz2 = iz * iz, iz3 = iz2 * iz;
    const float dtx = dj02 * (-f.fx * iz2), dty = dj12 * (-f.fy * iz2);
    float dtz = dj00 * (-f.fx * iz2) + dj11 * (-f.fy * iz2) + dj02 * (2.f * f.fx * vp.tx * iz3) +
                dj12 * (2.f * f.fy * vp.ty * iz3);
    float dt[3] = {0.f, 0.f, 0.f};
    if (vp.cx) dtz += dtx * vp.sx * f.limx;
    else dt[0] += dtx;
    if (vp.cy) dtz += dty * vp.sy * f.limy;
    else dt[1] += dty;
    dtz += gr.depth[i];  // depth = view z
    dt[2] += dtz;
    for (int k = 0; k < 3; ++k) dm[k] += vm[4 * k] * dt[0] + vm[4 * k + 1] * dt[1] + vm[4 * k + 2] * dt[2];
    // 4. SH color
    if (s.shs && gr.shs) {
        V3 v = v3(m.x - s.campos[0], m.y - s.campos[1], m.z - s.campos[2]);
        const float len = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z), il = 1.f / len;
        const V3 d = v3(v.x * il, v.y * il, v.z * il);
        float bs[16], bg[16][3];
        sh_basis(f.deg, d, bs);
        sh_basis_grad(f.deg, d, bg);
        const int nb = (f.deg + 1) * (f.deg + 1);
        float gcol[3];
        for (int ch = 0; ch < 3; ++ch) gcol[ch] = g.clamped[3 * i + ch] ? 0.f : gr.colors[3 * i + ch];
        float gdir[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < nb; ++k) {
            float proj = 0.f;
            for (int ch = 0; ch < 3; ++ch) {
                const float shv = s.shs[((long long)i * f.M + k) * 3 + ch];
                gr.shs[((long long)i * f.M + k) * 3 + ch] = bs[k] * gcol[ch];
                proj += shv * gcol[ch];
            }
            for (int a = 0; a < 3; ++a) gdir[a] += bg[k][a] * proj;
        }
        // d = v / |v|: dL/dv = (gdir - d (d . gdir)) / |v|
        const float dd = d.x * gdir[0] + d.y * gdir[1] + d.z * gdir[2];
        dm[0] += (gdir[0] - d.x * dd) * il;
        dm[1] += (gdir[1] - d.y * dd) * il;
        dm[2] += (gdir[2] - d.z * dd) * il;
    }
    for (int k = 0; k < 3; ++k) gr.means3D[3 * i + k] = dm[k];
    // 5. scale/rotation: Sigma = M^T M, M = S R^T; the normal is a signed column of R
    if (s.scales && s.rotations && (gr.scales || gr.rotations) && (!s.cov3D || !s.norm3D)) {
        const float* q = s.rotations + 4 * i;
        const float* sc = s.scales + 3 * i;
        float R[9], dR[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, dsc[3] = {0.f, 0.f, 0.f};
        quat_rot(q, R);
        if (!s.cov3D) {
            float Mx[9], dM[9];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) Mx[3 * r + c] = f.mod * sc[r] * R[3 * c + r];
            // dL/dM = 2 M dS (dS symmetric)
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c)
                    dM[3 * r + c] = 2.f * (Mx[3 * r] * dS[c] + Mx[3 * r + 1] * dS[3 + c] + Mx[3 * r + 2] * dS[6 + c]);
            // M[r][c] = mod s_r R[c][r]
            for (int r = 0; r < 3; ++r) {
                dsc[r] = f.mod * (dM[3 * r] * R[r] + dM[3 * r + 1] * R[3 + r] + dM[3 * r + 2] * R[6 + r]);
                for (int c = 0; c < 3; ++c) dR[3 * c + r] = dM[3 * r + c] * f.mod * sc[r];
            }
        }
        if (gr.scales)
            for (int r = 0; r < 3; ++r) gr.scales[3 * i + r] = dsc[r];
        if (!s.norm3D) {
            const int a = normal_axis(sc);
            // the stored normal is +/- column a of R; the exact adjoint takes
            // that sign, the reference's backward (backward.cu:364-366) the
            // sign of the stored normal against row a
            const float b0 = s.exact_adjoint ? R[a] : R[3 * a], b1 = s.exact_adjoint ? R[3 + a] : R[3 * a + 1],
                        b2 = s.exact_adjoint ? R[6 + a] : R[3 * a + 2];
            const float sgn = (g.normal[3 * i] * b0 + g.normal[3 * i + 1] * b1 + g.normal[3 * i + 2] * b2) < 0.f
                                  ? -1.f
                                  : 1.f;
            for (int c = 0; c < 3; ++c) dR[3 * c + a] += sgn * gr.norm3D[3 * i + c];
        }
        if (!gr.rotations) return;
        const float r = q[0], x = q[1], y = q[2], z = q[3];
        gr.rotations[4 * i] = 2.f * (-z * dR[1] + y * dR[2] + z * dR[3] - x * dR[5] - y * dR[6] + x * dR[7]);
        gr.rotations[4 * i + 1] =
            2.f * (y * dR[1] + z * dR[2] + y * dR[3] - 2.f * x * dR[4] - r * dR[5] + z * dR[6] + r * dR[7] - 2.f * x * dR[8]);
        gr.rotations[4 * i + 2] =
            2.f * (-2.f * y * dR[0] + x * dR[1] + r * dR[2] + x * dR[3] + z * dR[5] - r * dR[6] + z * dR[7] - 2.f * y * dR[8]);
        gr.rotations[4 * i + 3] =
            2.f * (-2.f * z * dR[0] - r * dR[1] + x * dR[2] + r * dR[3] - 2.f * z * dR[4] + y * dR[5] + x * dR[6] + y * dR[7]);
    }
}

template <typename Fn>
void with_ed(int ed, Fn&& fn)
{
    if (ed <= 0) fn(std::integral_constant<int, 0>());
    else if (ed <= 8) fn(std::integral_constant<int, 8>());
    else fn(std::integral_constant<int, GS_MAX_EXTRA>());
}

int fail_gs(int code, const char* msg)
{
    set_last_error(msg);
    return code;
}

bool check_scene(const GsScene* s)
{
    if (!s || s->P < 0 || s->H <= 0 || s->W <= 0 || !(s->tanfovx > 0.f) || !(s->tanfovy > 0.f)) return false;
    if (!s->bg || !s->viewmatrix || !s->projmatrix || !s->campos) return false;
    if (s->P > 0 && (!s->means3D || !s->opacities)) return false;
    if (s->P > 0 && !s->colors && (!s->shs || s->sh_degree < 0 || s->sh_degree > 3 ||
                                    s->sh_coeffs < (s->sh_degree + 1) * (s->sh_degree + 1)))
        return false;
    if (s->P > 0 && !s->cov3D && (!s->scales || !s->rotations)) return false;
    if (s->P > 0 && !s->norm3D && (!s->scales || !s->rotations)) return false;
    if (s->extra_dims < 0 || s->extra_dims > GS_MAX_EXTRA || (s->extra_dims > 0 && s->P > 0 && !s->extra)) return false;
    return true;
}

}  // namespace
}  // namespace mpm

using namespace mpm;

extern "C" int gs_scratch_bytes(int P, int L, int tiles, size_t* scan_bytes, size_t* sort_bytes)
{
    if (P < 0 || L < 0 || tiles < 0) return fail_gs(MPM_ERR_ARG, "gs_scratch_bytes: negative size");
    size_t a = 0, b = 0;
    int bits = 0;
    while ((1ll << bits) < (long long)tiles + 1) ++bits;
    cub::DeviceScan::InclusiveSum(nullptr, a, (uint32_t*)nullptr, (uint32_t*)nullptr, P > 0 ? P : 1);
    cub::DeviceRadixSort::SortPairs(nullptr, b, (uint64_t*)nullptr, (uint64_t*)nullptr, (uint32_t*)nullptr,
                                    (uint32_t*)nullptr, L > 0 ? L : 1, 0, 32 + bits);
    if (scan_bytes) *scan_bytes = a;
    if (sort_bytes) *sort_bytes = b;
    return MPM_OK;
}

extern "C" int gs_preprocess(const GsScene* s, const GsGeom* g, void* scan_tmp, size_t scan_bytes, int* num_rendered,
                             void* stream)
{
    if (!check_scene(s) || !g || !num_rendered) return fail_gs(MPM_ERR_ARG, "gs_preprocess: invalid argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    *num_rendered = 0;
    if (s->P == 0) return MPM_OK;
    const Frame f = make_frame(*s);
    k_gs_preprocess<<<(s->P + 255) / 256, 256, 0, st>>>(f, *s, *g);
    ++g_launches;
    size_t need = scan_bytes;
    if (cub::DeviceScan::InclusiveSum(scan_tmp, need, g->tiles_touched, g->offsets, s->P, st) != cudaSuccess)
        return fail_gs(MPM_ERR_CUDA, "gs_preprocess: prefix sum failed (scratch too small?)");
    uint32_t total = 0;
    if (cudaMemcpyAsync(&total, g->offsets + s->P - 1, sizeof total, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return fail_gs(MPM_ERR_CUDA, "gs_preprocess: CUDA error");
    if (total > 0x7fffffffu) return fail_gs(MPM_ERR_SHAPE, "gs_preprocess: too many tile overlaps");
    *num_rendered = (int)total;
    return MPM_OK;
}

extern "C" int gs_render(const GsScene* s, const GsGeom* g, int L, const GsBinning* b, void* sort_tmp,
                         size_t sort_bytes, const GsImage* img, void* stream)
{
    if (!check_scene(s) || !g || !b || !img || L < 0 || !img->color || !img->depth || !img->normal || !img->alpha ||
        !img->n_contrib || (s->extra_dims > 0 && !img->extra))
        return fail_gs(MPM_ERR_ARG, "gs_render: invalid argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const Frame f = make_frame(*s);
    const int tiles = f.gx * f.gy;
    if (cudaMemsetAsync(b->ranges, 0, sizeof(uint32_t) * 2 * (size_t)tiles, st) != cudaSuccess)
        return fail_gs(MPM_ERR_CUDA, "gs_render: memset failed");
    if (L > 0) {
        k_gs_duplicate<<<(s->P + 255) / 256, 256, 0, st>>>(f, *g, b->keys, b->ids);
        ++g_launches;
        int bits = 0;
        while ((1ll << bits) < (long long)tiles + 1) ++bits;
        size_t need = sort_bytes;
        if (cub::DeviceRadixSort::SortPairs(sort_tmp, need, b->keys, b->keys_sorted, b->ids, b->ids_sorted, L, 0,
                                            32 + bits, st) != cudaSuccess)
            return fail_gs(MPM_ERR_CUDA, "gs_render: sort failed (scratch too small?)");
        k_gs_ranges<<<(L + 255) / 256, 256, 0, st>>>(L, b->keys_sorted, b->ranges);
        ++g_launches;
    }
    const dim3 grid(f.gx, f.gy), block(kT, kT);
    with_ed(f.ED, [&](auto ed) {
        k_gs_render<decltype(ed)::value><<<grid, block, 0, st>>>(f, *s, *g, b->ids_sorted, b->ranges, *img);
    });
    ++g_launches;
    if (cudaGetLastError() != cudaSuccess) return fail_gs(MPM_ERR_CUDA, "gs_render: launch failed");
    return MPM_OK;
}

extern "C" int gs_backward(const GsScene* s, const GsGeom* g, int L, const GsBinning* b, const GsImage* img,
                           const float* dL_dcolor, const float* dL_ddepth, const float* dL_dnormal,
                           const float* dL_dalpha, const float* dL_dextra, const GsGrads* out, void* stream)
{
    if (!check_scene(s) || !g || !b || !img || !out || L < 0 || !out->means3D || !out->means2D || !out->opacities ||
        !out->colors || !out->cov3D || !out->norm3D || !out->conic || !out->depth)
        return fail_gs(MPM_ERR_ARG, "gs_backward: invalid argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const Frame f = make_frame(*s);
    const size_t P = (size_t)s->P;
    struct Z {
        void* p;
        size_t n;
    } zs[] = {{out->means3D, 12 * P}, {out->means2D, 12 * P}, {out->opacities, 4 * P}, {out->colors, 12 * P},
              {out->cov3D, 24 * P}, {out->norm3D, 12 * P}, {out->conic, 12 * P}, {out->depth, 4 * P},
              {out->shs, out->shs ? 12 * P * (size_t)s->sh_coeffs : 0}, {out->scales, out->scales ? 12 * P : 0},
              {out->rotations, out->rotations ? 16 * P : 0},
              {out->extra, out->extra ? 4 * P * (size_t)s->extra_dims : 0}};
    for (const Z& z : zs)
        if (z.p && z.n && cudaMemsetAsync(z.p, 0, z.n, st) != cudaSuccess)
            return fail_gs(MPM_ERR_CUDA, "gs_backward: memset failed");
    if (s->P == 0) return MPM_OK;
    const dim3 grid(f.gx, f.gy), block(kT, kT);
    with_ed(f.ED, [&](auto ed) {
        constexpr int E = decltype(ed)::value;
        const bool hd = dL_ddepth != nullptr, hn = dL_dnormal != nullptr;
        if (hd && hn)
            k_gs_render_bwd<E, true, true><<<grid, block, 0, st>>>(f, *s, *g, b->ids_sorted, b->ranges, *img,
                                                                   dL_dcolor, dL_ddepth, dL_dnormal, dL_dalpha,
                                                                   dL_dextra, *out);
        else if (hd)
            k_gs_render_bwd<E, true, false><<<grid, block, 0, st>>>(f, *s, *g, b->ids_sorted, b->ranges, *img,
                                                                    dL_dcolor, dL_ddepth, dL_dnormal, dL_dalpha,
                                                                    dL_dextra, *out);
        else if (hn)
            k_gs_render_bwd<E, false, true><<<grid, block, 0, st>>>(f, *s, *g, b->ids_sorted, b->ranges, *img,
                                                                    dL_dcolor, dL_ddepth, dL_dnormal, dL_dalpha,
                                                                    dL_dextra, *out);
        else
            k_gs_render_bwd<E, false, false><<<grid, block, 0, st>>>(f, *s, *g, b->ids_sorted, b->ranges, *img,
                                                                     dL_dcolor, dL_ddepth, dL_dnormal, dL_dalpha,
                                                                     dL_dextra, *out);
    });
    ++g_launches;
    k_gs_preprocess_bwd<<<(s->P + 255) / 256, 256, 0, st>>>(f, *s, *g, *out);
    ++g_launches;
    if (cudaGetLastError() != cudaSuccess) return fail_gs(MPM_ERR_CUDA, "gs_backward: launch failed");
    if (cudaStreamSynchronize(st) != cudaSuccess) return fail_gs(MPM_ERR_CUDA, "gs_backward: CUDA error");
    return MPM_OK;
}
