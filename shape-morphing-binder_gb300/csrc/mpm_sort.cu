// mpm_sort.cu -- particle order by grid cell for the re-sort of a graph's
// particles: at set-up (cell_order), and inside a rollout at the start of
// each checkpoint segment (cell_order_async, on preallocated scratch, so it
// can be recorded in a CUDA graph).
//
// The scatter and gather kernels are fastest when the particles of one block
// share few cells (segmented scatter, node tiles).  Particles drift between
// cells as a rollout runs, and a graph whose first layer is the last layer of
// an earlier rollout (promote_last_as_initial, as run.py does between
// episodes) starts out of order.  cell_order() computes the stable order of
// the particles by (instance, cell) with a CUB radix sort of 64-bit keys; the
// engine applies it to every particle plane and keeps the permutation, so the
// order callers see never changes.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <vector>

#include "mpm_launch.h"

namespace mpm {

namespace {

constexpr int kSortThreads = 256;
constexpr int kCellBits = 40;  // cell index bits of a key; the instance sits above

// key of slot p: (instance << cbits) | linear cell of the particle, clamped
// into the grid; padding slots (p >= n_valid) sort last within their instance
template <typename R>
__global__ void k_cell_keys(int p0, int count, int n_valid, long long ld, const R* __restrict__ x, int d0, int d1,
                            int d2, R g0, R g1, R g2, R inv_dx, unsigned long long inst,
                            unsigned long long* __restrict__ keys, int* __restrict__ vals, int cbits = kCellBits)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int p = p0 + t;
    unsigned long long cell = (1ull << cbits) - 1;
    if (t < n_valid) {
        const R xs[3] = {x[p], x[ld + p], x[2 * ld + p]};
        const R gm[3] = {g0, g1, g2};
        const int dm[3] = {d0, d1, d2};
        long long c[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const R f = (xs[a] - gm[a]) * inv_dx;
            // NaN and out-of-grid positions clamp to the grid's faces
            long long v = (f == f) ? (long long)floor(fmax(fmin(f, (R)(dm[a] - 1)), (R)0)) : 0;
            c[a] = v;
        }
        cell = ((unsigned long long)c[0] * (unsigned long long)d1 + (unsigned long long)c[1]) * (unsigned long long)d2 +
               (unsigned long long)c[2];
    }
    keys[p] = (inst << cbits) | cell;
    vals[p] = p;
}

// perm_new[i] = perm_old[order[i]] (order[i] itself without perm_old) and
// back[order[i]] = i, the slot in the new order of old slot order[i]
__global__ void k_perm_compose(int n, const int* __restrict__ order, const int* __restrict__ perm_old,
                               int* __restrict__ perm_new, int* __restrict__ back)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int o = order[i];
    perm_new[i] = perm_old ? perm_old[o] : o;
    back[o] = i;
}

// inv[perm[j]] = j
__global__ void k_perm_invert(int n, const int* __restrict__ perm, int* __restrict__ inv)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) inv[perm[j]] = j;
}

// rel[i] = inv_old[perm_new[i]] (perm_new[i] without inv_old): the slot in
// the old order of the particle the new order puts at slot i
__global__ void k_perm_rel(int n, const int* __restrict__ inv_old, const int* __restrict__ perm_new,
                           int* __restrict__ rel)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rel[i] = inv_old ? inv_old[perm_new[i]] : perm_new[i];
}

// bits of a cell key: every cell index of the grid and the padding value
// (all ones) above them
int cell_bits(const int* dims)
{
    const unsigned long long cells = (unsigned long long)dims[0] * dims[1] * dims[2];
    int b = 1;
    while (b < kCellBits && ((1ull << b) - 1) <= cells) ++b;
    return b;
}

struct Scratch {
    void* p = nullptr;
    explicit Scratch(size_t bytes)
    {
        if (bytes && cudaMalloc(&p, bytes) != cudaSuccess) p = nullptr;
    }
    ~Scratch()
    {
        if (p) cudaFree(p);
    }
};

}  // namespace

template <typename R>
bool cell_order(const StepCfg& c, const InstHost* inst, int ninst, int n, long long ld, const R* x, int* order,
                cudaStream_t s)
{
    if (n <= 0) return true;
    Scratch kin(sizeof(unsigned long long) * n), kout(sizeof(unsigned long long) * n), vin(sizeof(int) * n);
    if (!kin.p || !kout.p || !vin.p) return false;
    auto* keys = static_cast<unsigned long long*>(kin.p);
    auto* vals = static_cast<int*>(vin.p);
    int inst_bits = 0;
    if (ninst <= 0) {
        const int blocks = (n + kSortThreads - 1) / kSortThreads;
        k_cell_keys<R><<<blocks, kSortThreads, 0, s>>>(0, n, n, ld, x, c.dims[0], c.dims[1], c.dims[2], (R)c.gmin[0],
                                                       (R)c.gmin[1], (R)c.gmin[2], (R)(1.0 / c.dx), 0ull, keys, vals);
        ++g_launches;
    } else {
        while ((1 << inst_bits) < ninst) ++inst_bits;
        for (int i = 0; i < ninst; ++i) {
            const InstHost& h = inst[i];
            const long long end = i + 1 < ninst ? inst[i + 1].poff : n;
            const int count = (int)(end - h.poff);
            if (count <= 0) continue;
            const int blocks = (count + kSortThreads - 1) / kSortThreads;
            k_cell_keys<R><<<blocks, kSortThreads, 0, s>>>((int)h.poff, count, h.n, ld, x, h.dims[0], h.dims[1],
                                                           h.dims[2], (R)h.gmin[0], (R)h.gmin[1], (R)h.gmin[2],
                                                           (R)(1.0 / h.dx), (unsigned long long)i, keys, vals);
            ++g_launches;
        }
    }
    const int end_bit = kCellBits + inst_bits;
    size_t temp = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, temp, keys, static_cast<unsigned long long*>(kout.p), vals, order, n, 0,
                                    end_bit, s);
    Scratch tmp(temp);
    if (temp && !tmp.p) return false;
    if (cub::DeviceRadixSort::SortPairs(tmp.p, temp, keys, static_cast<unsigned long long*>(kout.p), vals, order, n,
                                        0, end_bit, s) != cudaSuccess)
        return false;
    return cudaStreamSynchronize(s) == cudaSuccess;  // scratch is freed on return
}

size_t SortWork::temp_for(int n)
{
    size_t temp = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, temp, (unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                    (int*)nullptr, (int*)nullptr, n, 0, 64);
    return temp;
}

template <typename R>
void cell_order_async(const StepCfg& c, const InstHost* inst, int ninst, int n, long long ld, const R* x,
                      int* order, const SortWork& w, cudaStream_t s)
{
    if (n <= 0) return;
    int cbits = 1, inst_bits = 0;
    if (ninst <= 0) {
        cbits = cell_bits(c.dims);
        const int blocks = (n + kSortThreads - 1) / kSortThreads;
        k_cell_keys<R><<<blocks, kSortThreads, 0, s>>>(0, n, n, ld, x, c.dims[0], c.dims[1], c.dims[2], (R)c.gmin[0],
                                                       (R)c.gmin[1], (R)c.gmin[2], (R)(1.0 / c.dx), 0ull, w.keys_in,
                                                       w.vals, cbits);
        ++g_launches;
    } else {
        for (int i = 0; i < ninst; ++i) cbits = std::max(cbits, cell_bits(inst[i].dims));
        while ((1 << inst_bits) < ninst) ++inst_bits;
        for (int i = 0; i < ninst; ++i) {
            const InstHost& h = inst[i];
            const long long end = i + 1 < ninst ? inst[i + 1].poff : n;
            const int count = (int)(end - h.poff);
            if (count <= 0) continue;
            const int blocks = (count + kSortThreads - 1) / kSortThreads;
            k_cell_keys<R><<<blocks, kSortThreads, 0, s>>>((int)h.poff, count, h.n, ld, x, h.dims[0], h.dims[1],
                                                           h.dims[2], (R)h.gmin[0], (R)h.gmin[1], (R)h.gmin[2],
                                                           (R)(1.0 / h.dx), (unsigned long long)i, w.keys_in,
                                                           w.vals, cbits);
            ++g_launches;
        }
    }
    size_t temp = w.temp_bytes;
    cub::DeviceRadixSort::SortPairs(w.temp, temp, w.keys_in, w.keys_out, w.vals, order, n, 0, cbits + inst_bits, s);
}

void launch_perm_compose(int n, const int* order, const int* perm_old, int* perm_new, int* back, cudaStream_t s)
{
    if (n <= 0) return;
    k_perm_compose<<<(n + kSortThreads - 1) / kSortThreads, kSortThreads, 0, s>>>(n, order, perm_old, perm_new,
                                                                                    back);
    ++g_launches;
}

void launch_perm_relative(int n, const int* perm_old, const int* perm_new, int* inv_scratch, int* rel,
                          cudaStream_t s)
{
    if (n <= 0) return;
    const int blocks = (n + kSortThreads - 1) / kSortThreads;
    if (perm_old) {
        k_perm_invert<<<blocks, kSortThreads, 0, s>>>(n, perm_old, inv_scratch);
        ++g_launches;
    }
    k_perm_rel<<<blocks, kSortThreads, 0, s>>>(n, perm_old ? inv_scratch : nullptr, perm_new, rel);
    ++g_launches;
}

template void cell_order_async<float>(const StepCfg&, const InstHost*, int, int, long long, const float*, int*,
                                      const SortWork&, cudaStream_t);
template void cell_order_async<double>(const StepCfg&, const InstHost*, int, int, long long, const double*, int*,
                                       const SortWork&, cudaStream_t);

template bool cell_order<float>(const StepCfg&, const InstHost*, int, int, long long, const float*, int*,
                                cudaStream_t);
template bool cell_order<double>(const StepCfg&, const InstHost*, int, int, long long, const double*, int*,
                                 cudaStream_t);

}  // namespace mpm
