// mpm_noalloc.cu -- an allocation-free variant of the end-layer mass loss.
//
// mpm_mass_loss_noalloc() computes the same loss and dL/dx as
// mpm_compgraph_mass_loss() (the EndLayerMassLoss path), for callers that
// hand in their own device buffers and cannot allocate device memory
// themselves or through this library: code that must stay inside a fixed
// device-memory budget it may not grow (a memory pool reserved up front), or
// a host runtime that owns every device allocation of the process.
// Its scratch (the grid mass, dL/dm per node and the four FP64 reduction
// accumulators) lives in one file-scope __device__ array.  The array belongs
// to this file's device code, which CUDA loads into a device's context when
// the first call on that device touches it (lazy module loading, the
// default): that first call allocates the module's memory, array included,
// and the memory stays until the context is destroyed.  Callers therefore
// make one call per device ahead of time, outside the restricted context
// (or run with CUDA_MODULE_LOADING=EAGER, which loads it with the library);
// later calls allocate nothing.  Every call shares the array: calls that
// overlap on the GPU (different streams or host threads without ordering)
// race and give wrong results.  The call is synchronous (it copies the loss
// back and waits for its stream), so it must not be made from a stream
// callback, and it refuses a stream that is being captured.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>

#include "../../include/mpm.h"
#include "mpm_launch.h"
#include "mpm_math.cuh"

namespace {

constexpr long long kMaxNodes = MPM_NOALLOC_MAX_NODES;
constexpr size_t kAccBytes = 256;  // 4 doubles, padded to the alignment
constexpr size_t kScratchBytes = kAccBytes + 2 * sizeof(float) * (size_t)kMaxNodes;

// layout: [acc: 4 doubles | pad][grid mass: kMaxNodes floats][dL/dm: kMaxNodes floats]
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct Geo {
    int dims[3];
    float dx, inv_dx;
    float gmin[3];
};

__device__ __forceinline__ bool inside(const Geo& g, int i, int j, int k)
{
    return (unsigned)i < (unsigned)g.dims[0] && (unsigned)j < (unsigned)g.dims[1] && (unsigned)k < (unsigned)g.dims[2];
}

__device__ __forceinline__ long long node(const Geo& g, int i, int j, int k)
{
    return ((long long)i * g.dims[1] + j) * g.dims[2] + k;
}

__global__ void k_nl_mass(Geo g, int n, const float* __restrict__ x, const float* __restrict__ m, float* gm)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
    mpm::Stencil<float, 4> st;
    mpm::make_stencil<float, 4>(xp, g.gmin, g.dx, g.inv_dx, st, false);
    const float mp = m[p];
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b)
            for (int c = 0; c < 4; ++c) {
                const int i = st.base[0] + a, j = st.base[1] + b, k = st.base[2] + c;
                if (inside(g, i, j, k)) atomicAdd(&gm[node(g, i, j, k)], st.w[0][a] * st.w[1][b] * st.w[2][c] * mp);
            }
}

__device__ double block_sum(double v, double* red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    }
    __syncthreads();
    return s;
}

__global__ void k_nl_sums(long long nn, const float* __restrict__ gm, const float* __restrict__ tm, double* acc)
{
    __shared__ double red[32];
    double a = 0, b = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x) {
        a += gm[i];
        b += tm[i];
    }
    a = block_sum(a, red);
    b = block_sum(b, red);
    if (threadIdx.x == 0) {
        atomicAdd(&acc[0], a);
        atomicAdd(&acc[1], b);
    }
}

// CompGraph.cpp:60-92: per-node log-mass loss and dL/dm
__global__ void k_nl_nodes(long long nn, const float* __restrict__ gm, const float* __restrict__ tm, float* dLdm,
                           double* acc)
{
    __shared__ double red[32];
    const double eps = 1e-4, min_mass = 1e-3, eps_s = 1e-6;
    const double sc = (acc[1] + eps_s) / (acc[0] + eps_s);
    double loss = 0, gc = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x) {
        const double c = gm[i], cms = sc * c;
        const double ld = log(cms + 1.0 + eps) - log((double)tm[i] + 1.0 + eps);
        loss += 0.5 * ld * ld;
        double gg = ld / (cms + 1.0 + eps);
        if (cms < min_mass) {
            const double diff = min_mass - cms;
            loss += diff * diff;
            gg += -2.0 * diff;
        }
        dLdm[i] = (float)(sc * gg);
        gc += gg * c;
    }
    loss = block_sum(loss, red);
    gc = block_sum(gc, red);
    if (threadIdx.x == 0) {
        atomicAdd(&acc[2], loss);
        atomicAdd(&acc[3], gc);
    }
}

// CompGraph.cpp:94-126: dL/dx per particle
__global__ void k_nl_grad(Geo g, int n, int exact, const float* __restrict__ x, const float* __restrict__ m,
                          const float* __restrict__ tm, const float* __restrict__ dLdm, const double* acc,
                          float* __restrict__ gx)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
    mpm::Stencil<float, 4> st;
    mpm::make_stencil<float, 4>(xp, g.gmin, g.dx, g.inv_dx, st, true);
    float corr = 0.f;
    if (exact) {
        const double sc = (acc[1] + 1e-6) / (acc[0] + 1e-6);
        corr = (float)(acc[3] * (-sc / (acc[0] + 1e-6)));
    }
    const float mp = m[p], nidx = -g.inv_dx;
    float a0 = 0, a1 = 0, a2 = 0;
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b)
            for (int c = 0; c < 4; ++c) {
                const int i = st.base[0] + a, j = st.base[1] + b, k = st.base[2] + c;
                if (!inside(g, i, j, k)) continue;
                const long long nd = node(g, i, j, k);
                const float pen = (exact || tm[nd] > 1e-12f) ? 1.f : 5.f;
                const float f = pen * mp * (dLdm[nd] + corr);
                a0 += f * nidx * st.s[0][a] * st.w[1][b] * st.w[2][c];
                a1 += f * nidx * st.w[0][a] * st.s[1][b] * st.w[2][c];
                a2 += f * nidx * st.w[0][a] * st.w[1][b] * st.s[2][c];
            }
    gx[3 * p] = a0;
    gx[3 * p + 1] = a1;
    gx[3 * p + 2] = a2;
}

int fail(int code, const char* msg)
{
    mpm::set_last_error(msg);
    return code;
}

}  // namespace

extern "C" int mpm_mass_loss_noalloc(int n, const float* x, const float* m, const float* target_mass,
                                     const int* dims, double dx, const double* min_point, int exact, float* dLdx,
                                     double* loss, void* stream)
{
    if (n < 0 || !dims || !loss || !(dx > 0) || (n > 0 && (!x || !m || !dLdx)) || !target_mass) {
        return fail(MPM_ERR_ARG, "mpm_mass_loss_noalloc: invalid argument");
    }
    if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) {
        return fail(MPM_ERR_ARG, "mpm_mass_loss_noalloc: grid dims must be positive");
    }
    const long long nn = (long long)dims[0] * dims[1] * dims[2];
    if (nn > kMaxNodes) {
        return fail(MPM_ERR_SHAPE, "mpm_mass_loss_noalloc: grid exceeds MPM_NOALLOC_MAX_NODES nodes");
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // synchronous call: refuse a stream under capture (the final stream
    // synchronize would fail and invalidate the caller's capture)
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return fail(MPM_ERR_STATE, "mpm_mass_loss_noalloc: the stream is being captured (the call is synchronous)");
    }
    // The host name of a __device__ array is not a device address.  The
    // address is looked up on every call, with the caller's device current:
    // it is only valid in the context the module is loaded into, which a
    // device reset or another current context replaces.
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) {
        return fail(MPM_ERR_CUDA, "mpm_mass_loss_noalloc: cudaGetSymbolAddress failed");
    }
    unsigned char* base = static_cast<unsigned char*>(ptr);
    double* acc = reinterpret_cast<double*>(base);
    float* gm = reinterpret_cast<float*>(base + kAccBytes);
    float* dLdm = gm + kMaxNodes;
    Geo g;
    for (int a = 0; a < 3; ++a) {
        g.dims[a] = dims[a];
        g.gmin[a] = (float)(min_point ? min_point[a] : 0.0);
    }
    g.dx = (float)dx;
    g.inv_dx = (float)(1.0 / dx);
    // the scratch keeps the previous call's contents: clear what accumulates
    if (cudaMemsetAsync(acc, 0, 4 * sizeof(double), s) != cudaSuccess ||
        cudaMemsetAsync(gm, 0, sizeof(float) * nn, s) != cudaSuccess) {
        return fail(MPM_ERR_CUDA, "mpm_mass_loss_noalloc: cudaMemsetAsync failed");
    }
    const int T = 256;
    if (n > 0) k_nl_mass<<<(n + T - 1) / T, T, 0, s>>>(g, n, x, m, gm);
    const int nb = (int)(nn + T - 1) / T < 1184 ? (int)((nn + T - 1) / T) : 1184;
    k_nl_sums<<<nb, T, 0, s>>>(nn, gm, target_mass, acc);
    k_nl_nodes<<<nb, T, 0, s>>>(nn, gm, target_mass, dLdm, acc);
    if (n > 0) k_nl_grad<<<(n + T - 1) / T, T, 0, s>>>(g, n, exact, x, m, target_mass, dLdm, acc, dLdx);
    double h[4];
    if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(h, acc, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        return fail(MPM_ERR_CUDA, "mpm_mass_loss_noalloc: CUDA error");
    }
    *loss = h[2];
    return MPM_OK;
}
