// mpm_launch.h -- host-side launchers for the MPM kernels (internal header).
//
// Particle state of one layer is stored as planes (structure of arrays) of
// length ld >= n:  x0..x2, v0..v2, C00..C22, F00..F22   (24 planes, STATE_*)
// Particle constants:  m, vol, lam, mu                  (4 planes,  CONST_*)
// Control dFc:          9 planes (absent = zero)
// Layer gradients:      dL/dx, dL/dv, dL/dF, dL/dC       (24 planes, same order)
// Grid nodes: 4 scalars per node, node (i,j,k) at (i*dy + j)*dz + k
//   forward grid: (p0,p1,p2,m) after P2G, (v0,v1,v2,m) after the grid update
//   adjoint grid: (dL/dv0..2, 0) after the G2P transpose, (dL/dp0..2, dL/dm)
//   after the grid-update transpose.
#pragma once
#include <cuda_runtime.h>

// 1: the grid update of a forward step clears the next step's grid and the
// grid adjoint of a backward step clears the next adjoint grid, instead of
// a separate memset pass per step
#ifndef MPM_FUSE_CLEAR
#define MPM_FUSE_CLEAR 1
#endif

namespace mpm {

enum { ST_X = 0, ST_V = 3, ST_C = 6, ST_F = 15, ST_N = 24 };
enum { CO_M = 0, CO_VOL = 1, CO_LAM = 2, CO_MU = 3, CO_N = 4 };

struct StepCfg {
    double dt = 1.0 / 120.0, drag = 0.5, smoothing = 0.1;
    double fext[3] = {0, 0, 0};
    double bulk = 0.25, jmin = 0.6;
    int dims[3] = {1, 1, 1};
    double dx = 1.0;
    double gmin[3] = {0, 0, 0};
    int kernel = 0;    // 0 cubic B-spline, 1 quadratic
    int material = 0;  // 0 fixed-corotated, 1 Neo-Hookean
    int exact = 0;     // 0 reference-compatible adjoint, 1 exact adjoint
    // batched launches: device table of InstDev<R> (one per instance) and the
    // total node count of the concatenated grids; null for one instance
    const void* inst = nullptr;
    int ninst = 0;
    long long total_nodes = 0;
    // per-graph tuning (-1: the process-wide defaults below).  tile_nodes is
    // the node-tile budget of P2G's scatter; adj_tile_nodes that of the G2P
    // transpose's scatter and gather_tile_nodes that of the P2G transpose's
    // gather (-1: tile_nodes).  Their best sizes differ: the G2P transpose
    // fits a fourth block per SM under 1024 nodes, the gather wants 2048+.
    int tile_nodes = -1;
    int scatter_mode = -1;
    int adj_tile_nodes = -1;
    int gather_tile_nodes = -1;
    // 1: a run of forward steps fuses each G2P with the next step's P2G
    // where the configuration allows it (g2p2g_applies); 0: step by step
    int fuse = 1;
    // threads (= particles) per block of the particle kernels of a step:
    // 256 or 128
    int threads = 256;
    // Deterministic scatters (FP32 segmented path): node sums accumulate in
    // 64-bit fixed point, so their value does not depend on the order of the
    // atomics.  fix: 4 words per node, all zero between steps (the grid
    // kernels that consume them clear them); fix_ctl: 4 words, [0] bits of
    // the largest particle mass, [1] bits of the largest |dL/dv_next|,
    // [2] bits of the largest |C0 dL/dC_next|, [3] overflow flags;
    // fix_scr: 12 particle planes (the G2P transpose's scatter inputs).
    // Scales are powers of two chosen so that every partial sum stays below
    // 2^62: mass from count * max m, momentum from that times fix_speed,
    // the adjoint from count * (max|dL/dv| + fix_reach * max|C0 dL/dC|).
    void* fix = nullptr;
    unsigned* fix_ctl = nullptr;
    float* fix_scr = nullptr;
    double fix_count = 0, fix_speed = 0, fix_reach = 0;
    long long nodes() const { return inst ? total_nodes : (long long)dims[0] * dims[1] * dims[2]; }
    bool det() const { return fix != nullptr; }
};

// partial sums of the deterministic reductions live after the first 8
// doubles of a reduction buffer: 8 + 2 * kRedParts doubles in all
constexpr int kRedParts = 1184;
constexpr size_t kRedDoubles = 8 + 2 * (size_t)kRedParts;

// host mirror of one batch instance (converted to the kernels' table)
struct InstHost {
    int dims[3];
    double dx, gmin[3];
    int n;
    long long poff, goff;
};
// builds the device table for precision R (sizeof(R) 4 or 8) into dst
void make_inst_table(const InstHost* h, int count, int kernel, int prec_bytes, void* dst, cudaStream_t s);
size_t inst_table_bytes(int count, int prec_bytes);

// Shared-memory tile budget (nodes) for the scatter kernels; 0 disables tiles.
extern int g_tile_nodes;
// nodes the P2G transpose stages per block unless the graph sets its budget
constexpr int kGatherTileDefault = 2048;
// FP32 scatter strategy: 1 = segmented (warp per cell segment, lane per
// node), 0 = per-particle scatter
extern int g_scatter_mode;
// fused G2P -> next P2G in forward passes (1, the default) or not (0)
extern int g_fuse_steps;
// kernels launched by the launchers below (host-side count)
extern long long g_launches;

template <typename R>
void launch_p2g(const StepCfg& c, int n, long long ld, const R* st, const R* dfc, const R* co, R* grid,
                cudaStream_t s);
template <typename R>
// zero_next (or null): a grid of nodes() nodes that the launch also clears
void launch_grid_update(const StepCfg& c, R* grid, cudaStream_t s, R* zero_next = nullptr);
template <typename R>
void launch_g2p(const StepCfg& c, int n, long long ld, const R* st, const R* dfc, const R* grid, R* st1, R* trust,
                cudaStream_t s);
// G2P of step i fused with P2G of step i+1 (FP32 segmented scatter, not
// deterministic): reads step i's updated grid, writes layer i+1 (st1, trust)
// and scatters layer i+1 into grid1 (zeroed).  g2p2g_applies: whether the
// configuration (precision, deterministic mode, scatter strategy) uses it.
bool g2p2g_applies(const StepCfg& c, int prec_bytes);
void launch_g2p2g(const StepCfg& c, int n, long long ld, const float* st, const float* dfc, const float* co,
                  const float* grid, float* st1, float* trust, float* grid1, cudaStream_t s);
// adjoint: G2P^T scatter (+P_op_2^T), grid update^T, P2G^T gather (+P_op_1^T)
template <typename R>
void launch_g2p_adj(const StepCfg& c, int n, long long ld, const R* st, const R* dfc, const R* st1, const R* g1,
                    const R* trust, R* adj, cudaStream_t s);
template <typename R>
// zero_next (or null): an adjoint grid that the launch also clears
void launch_grid_adj(const StepCfg& c, const R* grid, R* adj, cudaStream_t s, R* zero_next = nullptr);
template <typename R>
void launch_p2g_adj(const StepCfg& c, int n, long long ld, const R* st, const R* dfc, const R* co, const R* st1,
                    const R* g1, const R* trust, const R* grid, const R* adj, R* g, R* gFt, R* glam, R* gmu,
                    cudaStream_t s);

// mass loss (CompGraph.cpp:42-129).  target: a grid (4 scalars per node, mass
// in slot 3); acc: kRedDoubles doubles, results in the first 4 (sum_c,
// sum_t, loss, sum g*c), summed in a fixed order
template <typename R>
void launch_loss(const StepCfg& c, int n, long long ld, const R* st, const R* co, const R* target_m, R* gm, R* dLdm,
                 double* acc, R* g, cudaStream_t s);

// P2G with dt = drag = 0 into an un-reset grid, and the volume gather
template <typename R>
void launch_p2g_plain(const StepCfg& c, int n, long long ld, const R* st, const R* co, R* grid, cudaStream_t s);
template <typename R>
void launch_volumes(const StepCfg& c, int n, long long ld, const R* st, R* co, const R* grid, cudaStream_t s);

// Adam over one layer's control (PointCloud.cpp:83-147); sumsq of dL/dF
// into acc[0] (acc: kRedDoubles doubles, summed in a fixed order)
template <typename R>
void launch_sumsq(int n, long long ld, const R* g, int plane0, int planes, double* acc, cudaStream_t s);
template <typename R>
void launch_adam(int n, long long ld, const R* gF, R* dfc, double* mom, double* vec, double* vmax, double alpha,
                 double inv_gn, double beta1, double beta2, double eps, int t, cudaStream_t s);

// layout conversion: (n, k) row-major <-> k planes of stride ld; with perm,
// plane slot p holds row perm[p] of the caller's array
template <typename R, typename T>
void launch_aos_to_planes(int n, int k, long long ld, const T* src, R* dst, cudaStream_t s,
                          const int* perm = nullptr);
template <typename R, typename T>
void launch_planes_to_aos(int n, int k, long long ld, const R* src, T* dst, cudaStream_t s,
                          const int* perm = nullptr);
// k planes: dst slot i <- src slot order[i]
template <typename R>
void launch_gather_planes(int n, int k, long long ld, const int* order, const R* src, R* dst, cudaStream_t s);

// Particle order by (instance, grid cell), stable (mpm_sort.cu): order[i] is
// the slot whose particle moves to slot i.  x: 3 position planes of stride
// ld, precision R; inst/ninst: the batch (ninst 0: one instance described by
// c's grid).  Padding slots of a batch stay at the end of their instance.
// false: scratch allocation or sort failed (order not written).
template <typename R>
bool cell_order(const StepCfg& c, const InstHost* inst, int ninst, int n, long long ld, const R* x, int* order,
                cudaStream_t s);
// Scratch of an in-rollout re-sort (cell_order_async), allocated once per
// graph: keys, values and CUB's temporary storage for n slots
struct SortWork {
    unsigned long long* keys_in = nullptr;
    unsigned long long* keys_out = nullptr;
    int* vals = nullptr;
    void* temp = nullptr;
    size_t temp_bytes = 0;
    static size_t temp_for(int n);
};
// cell_order without allocations or synchronisation (stream-ordered, safe
// under stream capture)
template <typename R>
void cell_order_async(const StepCfg& c, const InstHost* inst, int ninst, int n, long long ld, const R* x,
                      int* order, const SortWork& w, cudaStream_t s);
// perm_new[i] = perm_old[order[i]] (perm_old null: order[i]); back[order[i]] = i
void launch_perm_compose(int n, const int* order, const int* perm_old, int* perm_new, int* back, cudaStream_t s);
// rel[i] = slot under perm_old of the particle perm_new puts at slot i
// (perm_old null: the identity); inv_scratch: n ints
void launch_perm_relative(int n, const int* perm_old, const int* perm_new, int* inv_scratch, int* rel,
                          cudaStream_t s);
template <typename R>
void launch_axpy_planes(int n, int k, long long ld, R alpha, const R* x, R* y, cudaStream_t s);
template <typename R>
void launch_fill_planes(int n, int k, long long ld, R value, R* y, cudaStream_t s);
// count of nonzero-mass nodes (for the roofline's active-node bytes)
template <typename R>
void launch_count_active(const StepCfg& c, const R* grid, unsigned long long* out, cudaStream_t s);
// non-finite check over planes; sets *flag = 1 on NaN/Inf
template <typename R>
void launch_nonfinite(int n, int k, long long ld, const R* y, int* flag, cudaStream_t s);

// deterministic mode: clear fix_ctl[0..2] and store the largest particle
// mass in fix_ctl[0] (start of every pass that scatters)
void launch_fix_prepare(const StepCfg& c, int n, long long ld, const float* co, cudaStream_t s);

// record the message mpm_last_error() returns on this host thread
void set_last_error(const char* msg);

}  // namespace mpm
