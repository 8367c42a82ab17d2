// mpm_geometry.cu -- inside test of mesh -> particle sampling on the GPU.
//
// GeometryLoading::GeneratePointCloudFromWatertightTriangleMesh
// (GeometryLoading.cpp:10-83) keeps the lattice points whose signed distance
// to the mesh is <= 0 under libigl's winding-number sign, i.e. the points
// with |generalized winding number| >= 1/2 and the points on the surface.
// k_winding computes the generalized winding number of every point: the sum
// over triangles of the signed solid angle (Van Oosterom & Strackee 1983,
// tan(Omega/2) = a.(b x c) / (|a||b||c| + (a.b)|c| + (a.c)|b| + (b.c)|a|))
// over 4 pi.  One thread per point; the triangles stream through shared
// memory in tiles, so every block reads each triangle once.  Per-tile sums
// are FP32, the running sum FP64.  A point on the surface (on a vertex, or
// in the plane of a triangle and inside it) gets w = 1/2 exactly, which the
// >= 1/2 rule keeps, as the reference's S <= 0 does for distance 0.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/mpm.h"
#include "mpm_launch.h"

namespace mpm {
namespace {

constexpr int kWThreads = 256;
constexpr int kWTile = 512;  // triangles per shared-memory tile (18 KB)

__global__ void __launch_bounds__(kWThreads) k_winding(int np, const float* __restrict__ pts, int nt,
                                                        const float* __restrict__ tri, double* __restrict__ w)
{
    __shared__ float st[kWTile * 9];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < np;
    float px = 0.f, py = 0.f, pz = 0.f;
    if (valid) {
        px = pts[3 * i];
        py = pts[3 * i + 1];
        pz = pts[3 * i + 2];
    }
    double acc = 0.0;
    bool on_surface = false;
    for (int t0 = 0; t0 < nt; t0 += kWTile) {
        const int cnt = min(kWTile, nt - t0);
        __syncthreads();
        for (int u = threadIdx.x; u < cnt * 9; u += blockDim.x) st[u] = tri[(long long)t0 * 9 + u];
        __syncthreads();
        if (!valid) continue;
        float sum = 0.f;
        for (int t = 0; t < cnt; ++t) {
            const float* q = st + t * 9;
            const float ax = q[0] - px, ay = q[1] - py, az = q[2] - pz;
            const float bx = q[3] - px, by = q[4] - py, bz = q[5] - pz;
            const float cx = q[6] - px, cy = q[7] - py, cz = q[8] - pz;
            const float la = sqrtf(ax * ax + ay * ay + az * az);
            const float lb = sqrtf(bx * bx + by * by + bz * bz);
            const float lc = sqrtf(cx * cx + cy * cy + cz * cz);
            const float num = ax * (by * cz - bz * cy) + ay * (bz * cx - bx * cz) + az * (bx * cy - by * cx);
            const float den = la * lb * lc + (ax * bx + ay * by + az * bz) * lc + (ax * cx + ay * cy + az * cz) * lb +
                              (bx * cx + by * cy + bz * cz) * la;
            if (la == 0.f || lb == 0.f || lc == 0.f || (num == 0.f && den <= 0.f)) on_surface = true;
            sum += atan2f(num, den);
        }
        acc += (double)sum;
    }
    if (valid) w[i] = on_surface ? 0.5 : acc / (2.0 * 3.14159265358979323846);
}

struct DevMem {
    void* p = nullptr;
    explicit DevMem(size_t b)
    {
        if (b && cudaMalloc(&p, b) != cudaSuccess) p = nullptr;
    }
    ~DevMem()
    {
        if (p) cudaFree(p);
    }
};

}  // namespace
}  // namespace mpm

extern "C" int mpm_winding_numbers(int n_points, const float* points, int n_tris, const float* tri_vertices,
                                   double* out, int on_device, void* stream)
{
    if (n_points < 0 || n_tris < 0 || (n_points > 0 && (!points || !out)) || (n_tris > 0 && !tri_vertices)) {
        mpm::set_last_error("mpm_winding_numbers: invalid argument");
        return MPM_ERR_ARG;
    }
    if (n_points == 0) return MPM_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const float* dp = points;
    const float* dt = tri_vertices;
    double* dw = out;
    mpm::DevMem mp(on_device ? 0 : sizeof(float) * 3 * (size_t)n_points);
    mpm::DevMem mt(on_device ? 0 : sizeof(float) * 9 * (size_t)n_tris);
    mpm::DevMem mw(on_device ? 0 : sizeof(double) * (size_t)n_points);
    if (!on_device) {
        if (!mp.p || (n_tris && !mt.p) || !mw.p) {
            mpm::set_last_error("mpm_winding_numbers: cudaMalloc failed");
            return MPM_ERR_OOM;
        }
        if (cudaMemcpyAsync(mp.p, points, sizeof(float) * 3 * (size_t)n_points, cudaMemcpyHostToDevice, s) !=
                cudaSuccess ||
            (n_tris && cudaMemcpyAsync(mt.p, tri_vertices, sizeof(float) * 9 * (size_t)n_tris, cudaMemcpyHostToDevice,
                                       s) != cudaSuccess)) {
            mpm::set_last_error("mpm_winding_numbers: host-to-device copy failed");
            return MPM_ERR_CUDA;
        }
        dp = static_cast<const float*>(mp.p);
        dt = static_cast<const float*>(mt.p);
        dw = static_cast<double*>(mw.p);
    }
    const int blocks = (n_points + mpm::kWThreads - 1) / mpm::kWThreads;
    mpm::k_winding<<<blocks, mpm::kWThreads, 0, s>>>(n_points, dp, n_tris, dt, dw);
    ++mpm::g_launches;
    if (cudaGetLastError() != cudaSuccess) {
        mpm::set_last_error("mpm_winding_numbers: launch failed");
        return MPM_ERR_CUDA;
    }
    if (!on_device &&
        cudaMemcpyAsync(out, dw, sizeof(double) * (size_t)n_points, cudaMemcpyDeviceToHost, s) != cudaSuccess) {
        mpm::set_last_error("mpm_winding_numbers: device-to-host copy failed");
        return MPM_ERR_CUDA;
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        mpm::set_last_error("mpm_winding_numbers: CUDA error");
        return MPM_ERR_CUDA;
    }
    return MPM_OK;
}
