// mpm_kernels.cu -- sm_103a kernels for the differentiable MPM step.
//
// Forward step (DiffMPMLib3D/ForwardSimulation.cpp:159-185) as three kernels:
//   k_p2g         P_op_1 + P2G: FCR stress fused into the momentum scatter,
//                 accumulated in a shared-memory node tile, flushed with few
//                 global atomics (ForwardSimulation.cpp:16-80)
//   k_grid_update mass clamp + G_op (ForwardSimulation.cpp:82-87,165-170)
//   k_g2p         G2P + P_op_2: velocity/affine gather, trust region,
//                 F update, smoothing, advection (ForwardSimulation.cpp:89-157)
// Adjoint step (DiffMPMLib3D/BackPropagation.cpp:9-144) as three kernels:
//   k_g2p_adj     P_op_2^T + G2P^T scatter of dL/dv_next, dL/dC_next
//   k_grid_adj    G_op^T per node
//   k_p2g_adj     P2G^T gather + stress VJP (P_op_1^T), matrix-free
// No kernel here uses tensor cores: nothing on this path is a dense
// contraction; the bound is memory traffic and FP32 issue rate.
#include <algorithm>
#include <climits>
#include <cstdint>
#include <unordered_map>
#include <vector>

#include "mpm_launch.h"
#include "mpm_math.cuh"

namespace mpm {

// resident blocks per SM the register allocator targets for the two
// heaviest kernels (compile-time tuning knobs)
#ifndef MPM_P2G_MIN_BLOCKS
#define MPM_P2G_MIN_BLOCKS 3
#endif
#ifndef MPM_P2G_ADJ_MIN_BLOCKS
#define MPM_P2G_ADJ_MIN_BLOCKS 1
#endif
#ifndef MPM_G2P_MIN_BLOCKS
#define MPM_G2P_MIN_BLOCKS 3
#endif
#ifndef MPM_G2P2G_MIN_BLOCKS
#define MPM_G2P2G_MIN_BLOCKS 3
#endif
// G2P of a step fused with the next step's P2G (FP32, segmented scatter)
#ifndef MPM_FUSE_G2P2G
#define MPM_FUSE_G2P2G 1
#endif

// scatter tiles off by default: the cell-group sums go straight to global
// memory as float4 reductions, faster than a shared tile and its flush on
// every workload measured; the gather tile has its own default
int g_tile_nodes = 0;
int g_scatter_mode = 1;
int g_fuse_steps = 1;
long long g_launches = 0;

namespace {

constexpr int kThreads = 256;

// One instance of a batch: its grid and its particle range.  Particle
// ranges start at multiples of the block size, so a block never straddles
// two instances.
template <typename R>
struct InstDev {
    R dx, inv_dx, C0, gmin[3];
    int dims[3];
    int n;
    long long poff, goff;
};

template <typename R>
struct KP {
    R dt, dragf, s, bulk, jmin, C0, dx, inv_dx;
    R gmin[3], dtf[3];
    int dims[3];
    int material, exact;
    const InstDev<R>* inst;  // null: one instance described by the fields above
    int ninst;
};

template <typename R>
KP<R> make_kp(const StepCfg& c)
{
    KP<R> k;
    k.dt = (R)c.dt;
    k.dragf = (R)(1.0 - c.dt * c.drag);
    k.s = (R)c.smoothing;
    k.bulk = (R)c.bulk;
    k.jmin = (R)c.jmin;
    k.C0 = (R)((c.kernel == 0 ? 3.0 : 4.0) / (c.dx * c.dx));
    k.dx = (R)c.dx;
    k.inv_dx = (R)(1.0 / c.dx);
    for (int a = 0; a < 3; ++a) {
        k.gmin[a] = (R)c.gmin[a];
        k.dtf[a] = (R)(c.dt * c.fext[a]);
        k.dims[a] = c.dims[a];
    }
    k.material = c.material;
    k.exact = c.exact;
    k.inst = static_cast<const InstDev<R>*>(c.inst);
    k.ninst = c.ninst;
    return k;
}

// Batched launches: point kp at the block's instance and return the end of
// its particle range and its first grid node.
template <typename R>
MPM_D void bind_instance(KP<R>& kp, int& n_end, long long& goff)
{
    goff = 0;
    if (!kp.inst) return;
    const long long p0 = (long long)blockIdx.x * blockDim.x;
    int lo = 0, hi = kp.ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (kp.inst[mid].poff <= p0) lo = mid;
        else hi = mid - 1;
    }
    const InstDev<R>& I = kp.inst[lo];
    kp.dx = I.dx;
    kp.inv_dx = I.inv_dx;
    kp.C0 = I.C0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        kp.gmin[a] = I.gmin[a];
        kp.dims[a] = I.dims[a];
    }
    n_end = (int)(I.poff + I.n);
    goff = I.goff;
}

inline int nblocks(long long n, int t = kThreads) { return (int)((n + t - 1) / t); }

// every kernel launch of the launchers below is counted (host side)
inline void counted() { ++g_launches; }

// select a[i] from a small register array without dynamic indexing
template <typename R, int K>
MPM_D R sel(const R (&a)[K], int i)
{
    R r = a[0];
#pragma unroll
    for (int q = 1; q < K; ++q) r = (i == q) ? a[q] : r;
    return r;
}

template <typename R>
MPM_D void load_planes(const R* __restrict__ base, long long ld, int p, int k, R* out)
{
#pragma unroll
    for (int i = 0; i < k; ++i) out[i] = base[(long long)i * ld + p];
}

template <typename R>
MPM_D void store_planes(R* __restrict__ base, long long ld, int p, int k, const R* v)
{
#pragma unroll
    for (int i = 0; i < k; ++i) base[(long long)i * ld + p] = v[i];
}

template <typename R>
MPM_D bool in_grid(const KP<R>& kp, int i, int j, int k)
{
    return (unsigned)i < (unsigned)kp.dims[0] && (unsigned)j < (unsigned)kp.dims[1] && (unsigned)k < (unsigned)kp.dims[2];
}

template <typename R>
MPM_D long long node_of(const KP<R>& kp, int i, int j, int k)
{
    return ((long long)i * kp.dims[1] + j) * kp.dims[2] + k;
}

// Ft = F + dFc
template <typename R>
MPM_D void load_Ft(const R* st, const R* dfc, long long ld, int p, R* F, R* Ft)
{
    load_planes(st + ST_F * ld, ld, p, 9, F);
    if (dfc) {
#pragma unroll
        for (int i = 0; i < 9; ++i) Ft[i] = F[i] + dfc[(long long)i * ld + p];
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i) Ft[i] = F[i];
    }
}

// ------------------------------------------------------------------------
// Scatter machinery shared by P2G (4 components: p0,p1,p2,m) and the G2P
// transpose (3 components: dL/dv).  A block owns a contiguous chunk of
// particles; when the chunk's stencil bounding box fits the shared tile
// budget, contributions are accumulated with shared-memory atomics and
// flushed once, otherwise they go straight to global atomics.  Each lane
// starts its walk over the stencil at a different (b,c) so lanes of one cell
// rarely hit the same node in the same instruction.
// ------------------------------------------------------------------------

template <typename R, int K, int NC>
struct Scatter {
    int b0, b1, b2, e0, e1, e2;
    bool tile;
    R* sm;
    int vol;

    MPM_D void setup(bool valid, const int* base, void* smem, int tile_cap)
    {
        __shared__ int box[6];
        if (threadIdx.x < 3) box[threadIdx.x] = INT_MAX;
        else if (threadIdx.x < 6) box[threadIdx.x] = INT_MIN;
        __syncthreads();
        tile = false;
        if (tile_cap > 0) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                int lo = valid ? base[a] : INT_MAX;
                int hi = valid ? base[a] : INT_MIN;
                lo = __reduce_min_sync(0xffffffffu, lo);
                hi = __reduce_max_sync(0xffffffffu, hi);
                if ((threadIdx.x & 31) == 0) {
                    atomicMin(&box[a], lo);
                    atomicMax(&box[3 + a], hi);
                }
            }
        }
        __syncthreads();
        if (tile_cap > 0 && box[0] != INT_MAX) {
            b0 = box[0];
            b1 = box[1];
            b2 = box[2];
            long long x0 = (long long)box[3] - box[0] + K, x1 = (long long)box[4] - box[1] + K,
                      x2 = (long long)box[5] - box[2] + K;
            // each extent is checked first so the product cannot overflow
            // (positions that are Inf/NaN give extents near 2^32)
            const bool small = x0 > 0 && x1 > 0 && x2 > 0 && x0 <= tile_cap && x1 <= tile_cap && x2 <= tile_cap;
            const long long v = small ? x0 * x1 * x2 : (long long)tile_cap + 1;
            if (v <= tile_cap) {
                tile = true;
                e0 = (int)x0;
                e1 = (int)x1;
                e2 = (int)x2;
                vol = (int)v;
                sm = reinterpret_cast<R*>(smem);
                for (int t = threadIdx.x; t < NC * vol; t += blockDim.x) sm[t] = R(0);
            }
        }
        __syncthreads();
    }

    MPM_D void add(const KP<R>& kp, R* __restrict__ grid, int i, int j, int k, const R* val)
    {
        if (tile) {
            int idx = ((i - b0) * e1 + (j - b1)) * e2 + (k - b2);
#pragma unroll
            for (int q = 0; q < NC; ++q) atomicAdd(&sm[q * vol + idx], val[q]);
        } else if (in_grid(kp, i, j, k)) {
            long long nd = node_of(kp, i, j, k);
#pragma unroll
            for (int q = 0; q < NC; ++q) atomicAdd(&grid[nd * 4 + q], val[q]);
        }
    }

    MPM_D void flush(const KP<R>& kp, R* __restrict__ grid)
    {
        __syncthreads();
        if (!tile) return;
        for (int t = threadIdx.x; t < vol; t += blockDim.x) {
            R v[NC];
            bool any = false;
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                v[q] = sm[q * vol + t];
                any |= (v[q] != R(0));
            }
            if (!any) continue;
            int kk = t % e2, r = t / e2;
            int jj = r % e1, ii = r / e1;
            int i = b0 + ii, j = b1 + jj, k = b2 + kk;
            if (!in_grid(kp, i, j, k)) continue;
            long long nd = node_of(kp, i, j, k);
#pragma unroll
            for (int q = 0; q < NC; ++q)
                if (v[q] != R(0)) atomicAdd(&grid[nd * 4 + q], v[q]);
        }
    }
};

// Walk the K^3 stencil, calling f(i, j, k, w, dg) with a lane-dependent order.
template <typename R, int K, typename Fn>
MPM_D void walk_rotated(const Stencil<R, K>& st, Fn&& f)
{
    const int lane = threadIdx.x & 31;
    const int rb = (lane >> 2) % K, rc = lane % K;
#pragma unroll
    for (int a = 0; a < K; ++a) {
        const R wa = st.w[0][a], ga = st.g[0][a];
#pragma unroll
        for (int bb = 0; bb < K; ++bb) {
            int b = bb + rb;
            b = b >= K ? b - K : b;
            const R wab = wa * sel(st.w[1], b), gb = sel(st.g[1], b);
#pragma unroll
            for (int cc = 0; cc < K; ++cc) {
                int c = cc + rc;
                c = c >= K ? c - K : c;
                const R w = wab * sel(st.w[2], c), gc = sel(st.g[2], c);
                f(st.base[0] + a, st.base[1] + b, st.base[2] + c, w, ga, gb, gc);
            }
        }
    }
}

// ------------------------------------------------------------------------
// Segmented scatter (FP32).  Particles arrive sorted by cell, so runs of
// particles share one stencil base.  Each block stages its chunk of
// particles as records in shared memory and splits the chunk into segments
// of equal base; a warp takes one segment at a time and each lane owns fixed
// stencil nodes (lane and lane+32), summing the segment's contributions in
// registers.  One shared atomic per node per segment replaces one per node
// per particle, and no two lanes of a warp touch the same node.  The node
// tile is then flushed to global memory once per block.  The contribution
// of particle p to node n is  w_pn * [u0_p + A_p dg_pn, (m_p)].
// ------------------------------------------------------------------------

constexpr int kRec = 40;  // u0[3], m, A[9], pad[3], (w, g) pairs [3][K<=4]

inline size_t seg_smem_bytes(int CH, int tile_cap, int NC, bool det = false)
{
    return (size_t)CH * kRec * 4 + (size_t)tile_cap * NC * (det ? 8 : 4);
}

// Deterministic accumulation.  A value y is added to a node as the integer
// round(y * 2^e) (two's complement in 64 bits); integer addition is
// associative, so the node sum does not depend on the order in which blocks,
// warps and cell groups deliver their contributions.  e is chosen per launch
// from a bound B on the sum of |contributions| of the launch so that
// B * 2^e < 2^62: no partial sum can wrap.  Resolution 2^-e = B * 2^-62 is
// far below FP32 rounding of the node values for any realistic particle
// count (2^21 particles leave 41 bits below the largest contribution).
struct FixArgs {
    unsigned long long* acc;  // 4 per node
    unsigned* ctl;            // see StepCfg::fix_ctl
    float count, speed, reach;
};

FixArgs make_fix(const StepCfg& c)
{
    FixArgs f;
    f.acc = static_cast<unsigned long long*>(c.fix);
    f.ctl = c.fix_ctl;
    f.count = (float)c.fix_count;
    f.speed = (float)c.fix_speed;
    f.reach = (float)c.fix_reach;
    return f;
}

// 2^e for -126 <= e <= 127, from the bit pattern
MPM_D float pow2f(int e) { return __int_as_float((e + 127) << 23); }

// e with bound * 2^e < 2^62 (bound < 2^(E+1) for the binary exponent E of
// bound), clamped to +-120; 0 for a zero or NaN bound
MPM_D int fix_exponent(float bound)
{
    if (!(bound > 0.f)) return 0;
    const int E = (int)((__float_as_uint(bound) >> 23) & 0xFF) - 127;
    return max(-120, min(120, 61 - E));
}

MPM_D float fix_mass_bound(const FixArgs& f) { return f.count * __uint_as_float(f.ctl[0]); }
MPM_D float fix_adj_bound(const FixArgs& f)
{
    return f.count * (__uint_as_float(f.ctl[1]) + f.reach * __uint_as_float(f.ctl[2]));
}

// y * 2^e rounded to an integer; flags values at or beyond 2^61 (and NaN)
MPM_D unsigned long long to_fix(float y, float scale, bool& ovf)
{
    const float z = y * scale;
    ovf |= !(fabsf(z) < 0x1p61f);
    return (unsigned long long)__float2ll_rn(z);
}

// Adds NC channel sums to a 16-byte grid node as one vector reduction
// (sm_90+).  With 3 channels (the adjoint grid's dL/dv, zeroed before the
// scatter) the fourth lane adds zero to a channel the scatter leaves free.
template <int NC>
MPM_D void add_node(float* node, const float* v)
{
    static_assert(NC == 3 || NC == 4, "grid nodes hold 4 floats");
    atomicAdd(reinterpret_cast<float4*>(node), make_float4(v[0], v[1], v[2], NC == 4 ? v[NC - 1] : 0.f));
}

template <int K, int NC, bool DET = false>
__device__ void seg_scatter(const KP<float>& kp, bool valid, const Stencil<float, K>& st, const float* u0, float m,
                            const float* A, float* __restrict__ grid, int tile_cap, unsigned char* smem,
                            const FixArgs* fx = nullptr, const float* scale = nullptr)
{
    const int CH = blockDim.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
    float* recs = reinterpret_cast<float*>(smem);
    float* tilebuf = recs + (size_t)CH * kRec;
    unsigned long long* tilefix = reinterpret_cast<unsigned long long*>(tilebuf);
    bool ovf = false;
    __shared__ int box[6];
    // Without a node tile (tile_cap 0, uniform over the launch) a warp reads
    // only its own lanes' records: no block-wide bounding box and no block
    // barriers, only the warp's own.
    const bool blockwide = tile_cap > 0;
    // 1. this lane's record, the block's bounding box of stencil bases
    if (blockwide) {
        if (t < 3) box[t] = INT_MAX;
        else if (t < 6) box[t] = INT_MIN;
    }
    if (valid) {
        float* r = recs + (size_t)t * kRec;
        r[0] = u0[0];
        r[1] = u0[1];
        r[2] = u0[2];
        r[3] = m;
#pragma unroll
        for (int i = 0; i < 9; ++i) r[4 + i] = A[i];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int o = 0; o < K; ++o) {
                r[16 + 2 * (a * K + o)] = st.w[a][o];
                r[17 + 2 * (a * K + o)] = st.g[a][o];
            }
    }
    if (blockwide) {
        __syncthreads();
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int lo = __reduce_min_sync(0xffffffffu, valid ? st.base[a] : INT_MAX);
            const int hi = __reduce_max_sync(0xffffffffu, valid ? st.base[a] : INT_MIN);
            if (lane == 0) {
                atomicMin(&box[a], lo);
                atomicMax(&box[3 + a], hi);
            }
        }
    } else {
        __syncwarp();
    }
    // 2. groups of lanes sharing a stencil base (not necessarily contiguous:
    //    particles drift across cells between sorts)
    const unsigned long long key =
        valid ? (((unsigned long long)(st.base[0] & 0x1FFFFF) << 42) |
                 ((unsigned long long)(st.base[1] & 0x1FFFFF) << 21) | (unsigned long long)(st.base[2] & 0x1FFFFF))
              : ~0ull;
    const unsigned grp = __match_any_sync(0xffffffffu, key);
    unsigned todo = __ballot_sync(0xffffffffu, valid);
    if (blockwide) __syncthreads();
    // 3. node tile over the bounding box, if it fits
    bool tile = false;
    int b0 = 0, b1 = 0, b2 = 0, e1 = 0, e2 = 0, vol = 0;
    if (blockwide && box[0] != INT_MAX) {
        const long long x0 = (long long)box[3] - box[0] + K, x1 = (long long)box[4] - box[1] + K,
                        x2 = (long long)box[5] - box[2] + K;
        if (x0 > 0 && x1 > 0 && x2 > 0 && x0 <= tile_cap && x1 <= tile_cap && x2 <= tile_cap &&
            x0 * x1 * x2 <= tile_cap) {
            tile = true;
            b0 = box[0];
            b1 = box[1];
            b2 = box[2];
            e1 = (int)x1;
            e2 = (int)x2;
            vol = (int)(x0 * x1 * x2);
            if constexpr (DET) {
                for (int i = t; i < NC * vol; i += CH) tilefix[i] = 0ull;
            } else {
                for (int i = t; i < NC * vol; i += CH) tilebuf[i] = 0.f;
            }
        }
    }
    if (blockwide) __syncthreads();
    // 4. each warp walks its cell groups, summing each group's contributions
    //    to the nodes a lane owns in registers, then deposits the sums
    const float* wrec = recs + (size_t)(warp * 32) * kRec;
    auto deposit = [&](int i, int j, int k, const float* acc) {
        if constexpr (DET) {
            if (tile) {
                const int idx = ((i - b0) * e1 + (j - b1)) * e2 + (k - b2);
#pragma unroll
                for (int q = 0; q < NC; ++q)
                    if (acc[q] != 0.f) atomicAdd(&tilefix[q * vol + idx], to_fix(acc[q], scale[q], ovf));
            } else if (in_grid(kp, i, j, k)) {
                const long long nd = node_of(kp, i, j, k);
#pragma unroll
                for (int q = 0; q < NC; ++q)
                    if (acc[q] != 0.f) atomicAdd(&fx->acc[nd * 4 + q], to_fix(acc[q], scale[q], ovf));
            }
        } else if (tile) {
            const int idx = ((i - b0) * e1 + (j - b1)) * e2 + (k - b2);
#pragma unroll
            for (int q = 0; q < NC; ++q)
                if (acc[q] != 0.f) atomicAdd(&tilebuf[q * vol + idx], acc[q]);
        } else if (in_grid(kp, i, j, k)) {
            add_node<NC>(grid + node_of(kp, i, j, k) * 4, acc);
        }
    };
    // a lane owns stencil nodes lane and lane+32
    constexpr int NODES = K * K * K;
    const int n0 = lane, n1 = lane + 32;
    const int a0 = n0 / (K * K), bb = (n0 / K) % K, cc = n0 % K;
    const bool has0 = n0 < NODES, has1 = n1 < NODES;
    const int a1 = has1 ? n1 / (K * K) : 0;
    while (todo) {
        const int lead = __ffs(todo) - 1;
        const unsigned members = __shfl_sync(0xffffffffu, grp, lead);
        todo &= ~members;
        const int i0 = __shfl_sync(0xffffffffu, st.base[0], lead);
        const int j0 = __shfl_sync(0xffffffffu, st.base[1], lead);
        const int k0 = __shfl_sync(0xffffffffu, st.base[2], lead);
        float acc0[NC], acc1[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) acc0[q] = acc1[q] = 0.f;
        if (has0) {
            unsigned mm = members;
            while (mm) {
                const int p = __ffs(mm) - 1;
                mm &= mm - 1;
                const float* r = wrec + (size_t)p * kRec;
                const float4 q0 = *reinterpret_cast<const float4*>(r);
                const float4 qa = *reinterpret_cast<const float4*>(r + 4);
                const float4 qb = *reinterpret_cast<const float4*>(r + 8);
                const float a8 = r[12];
                // (w, g) of the lane's y and z stencil offsets: one 8-byte load each
                const float2 wgy = *reinterpret_cast<const float2*>(r + 16 + 2 * (K + bb));
                const float2 wgz = *reinterpret_cast<const float2*>(r + 16 + 2 * (2 * K + cc));
                const float wyz = wgy.x * wgz.x;
                const float gy = wgy.y, gz = wgz.y;
                // A row-major: (qa.x qa.y qa.z | qa.w qb.x qb.y | qb.z qb.w a8)
                const float c0 = q0.x + qa.y * gy + qa.z * gz;
                const float c1 = q0.y + qb.x * gy + qb.y * gz;
                const float c2 = q0.z + qb.w * gy + a8 * gz;
                {
                    const float2 wgx = *reinterpret_cast<const float2*>(r + 16 + 2 * a0);
                    const float w = wgx.x * wyz, gx = wgx.y;
                    acc0[0] += w * (c0 + qa.x * gx);
                    acc0[1] += w * (c1 + qa.w * gx);
                    acc0[2] += w * (c2 + qb.z * gx);
                    if (NC == 4) acc0[NC - 1] += w * q0.w;
                }
                if (has1) {
                    const float2 wgx = *reinterpret_cast<const float2*>(r + 16 + 2 * a1);
                    const float w = wgx.x * wyz, gx = wgx.y;
                    acc1[0] += w * (c0 + qa.x * gx);
                    acc1[1] += w * (c1 + qa.w * gx);
                    acc1[2] += w * (c2 + qb.z * gx);
                    if (NC == 4) acc1[NC - 1] += w * q0.w;
                }
            }
            deposit(i0 + a0, j0 + bb, k0 + cc, acc0);
            if (has1) deposit(i0 + a1, j0 + bb, k0 + cc, acc1);
        }
    }
    if (blockwide) __syncthreads();
    // 5. flush the tile
    if constexpr (DET) {
        if (__any_sync(0xffffffffu, ovf) && lane == 0) atomicOr(&fx->ctl[3], 1u);
        if (tile) {
            for (int u = t; u < vol; u += CH) {
                unsigned long long v[NC];
                bool any = false;
#pragma unroll
                for (int q = 0; q < NC; ++q) {
                    v[q] = tilefix[q * vol + u];
                    any |= v[q] != 0ull;
                }
                if (!any) continue;
                const int kk = u % e2, rr = u / e2;
                const int jj = rr % e1, ii = rr / e1;
                const int i = b0 + ii, j = b1 + jj, k = b2 + kk;
                if (!in_grid(kp, i, j, k)) continue;
                const long long nd = node_of(kp, i, j, k);
#pragma unroll
                for (int q = 0; q < NC; ++q)
                    if (v[q] != 0ull) atomicAdd(&fx->acc[nd * 4 + q], v[q]);
            }
        }
        return;
    }
    if (tile) {
        for (int u = t; u < vol; u += CH) {
            float v[NC];
            bool any = false;
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                v[q] = tilebuf[q * vol + u];
                any |= v[q] != 0.f;
            }
            if (!any) continue;
            const int kk = u % e2, rr = u / e2;
            const int jj = rr % e1, ii = rr / e1;
            const int i = b0 + ii, j = b1 + jj, k = b2 + kk;
            if (!in_grid(kp, i, j, k)) continue;
            add_node<NC>(grid + node_of(kp, i, j, k) * 4, v);
        }
    }
}

// ------------------------------------------------------------------ P2G

template <typename R, int K>
__global__ void __launch_bounds__(kThreads) k_p2g(KP<R> kp, int n, long long ld, const R* __restrict__ st,
                                                   const R* __restrict__ dfc, const R* __restrict__ co,
                                                   R* __restrict__ grid, int tile_cap)
{
    extern __shared__ __align__(16) unsigned char smem[];
    long long goff;
    bind_instance(kp, n, goff);
    grid += goff * 4;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < n;
    Stencil<R, K> sten;
    R A[9], mv[3], mass = R(0);
    if (valid) {
        R x[3], v[3], C[9], F[9], Ft[9];
        load_planes(st + ST_X * ld, ld, p, 3, x);
        load_planes(st + ST_V * ld, ld, p, 3, v);
        load_planes(st + ST_C * ld, ld, p, 9, C);
        load_Ft(st, dfc, ld, p, F, Ft);
        mass = co[CO_M * ld + p];
        const R vol = co[CO_VOL * ld + p], lam = co[CO_LAM * ld + p], mu = co[CO_MU * ld + p];
        Inv<R> iv;
        invariants(Ft, iv);
        R P[9], Rm[9], S[9], PF[9];
        pk(kp.material, Ft, lam, mu, iv, P, Rm, S);
        mulNT3(P, Ft, PF);
        const R trC = C[0] + C[4] + C[8];
        const R k1 = -kp.C0 * kp.dt * vol;
#pragma unroll
        for (int i = 0; i < 9; ++i) A[i] = k1 * (PF[i] + ((i % 4 == 0) ? kp.bulk * trC : R(0))) + mass * C[i];
#pragma unroll
        for (int a = 0; a < 3; ++a) mv[a] = mass * v[a] * kp.dragf;
        make_stencil<R, K>(x, kp.gmin, kp.dx, kp.inv_dx, sten, false);
    }
    Scatter<R, K, 4> sc;
    sc.setup(valid, sten.base, smem, tile_cap);
    if (valid) {
        walk_rotated<R, K>(sten, [&](int i, int j, int k, R w, R gx, R gy, R gz) {
            R val[4];
#pragma unroll
            for (int r = 0; r < 3; ++r) val[r] = w * (mv[r] + A[r * 3] * gx + A[r * 3 + 1] * gy + A[r * 3 + 2] * gz);
            val[3] = w * mass;
            sc.add(kp, grid, i, j, k, val);
        });
    }
    sc.flush(kp, grid);
}

// -------------------------------------------------------- grid update

template <typename R>
__global__ void k_grid_update(KP<R> kp, long long nn, R* __restrict__ grid, R* __restrict__ zero_next)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    if constexpr (sizeof(R) == 4) {
        // the next step's grid, cleared here instead of by a separate pass
        if (zero_next) reinterpret_cast<float4*>(zero_next)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        // one 16-byte load per node; a node whose update leaves its bits as
        // they are (every node no particle reached: all zero) is not written
        float4* g = reinterpret_cast<float4*>(grid) + i;
        const float4 q = *g;
        if (q.w > 1e-12f) {
            *g = make_float4(q.x / q.w + kp.dtf[0], q.y / q.w + kp.dtf[1], q.z / q.w + kp.dtf[2], q.w);
        } else if ((__float_as_uint(q.x) | __float_as_uint(q.y) | __float_as_uint(q.z)) != 0u || q.w < 0.f) {
            *g = make_float4(0.f, 0.f, 0.f, q.w < 0.f ? 0.f : q.w);
        }
        return;
    }
    if (zero_next) {
        R* z = zero_next + 4 * i;
        z[0] = z[1] = z[2] = z[3] = R(0);
    }
    R* g = grid + 4 * i;
    R m = g[3];
    if (m < R(0)) m = R(0);
    R v0 = 0, v1 = 0, v2 = 0;
    if (m > R(1e-12)) {
        v0 = g[0] / m + kp.dtf[0];
        v1 = g[1] / m + kp.dtf[1];
        v2 = g[2] / m + kp.dtf[2];
    }
    g[0] = v0;
    g[1] = v1;
    g[2] = v2;
    g[3] = m;
}

// load the 3 velocity components of node nd
template <typename R>
MPM_D void load_node3(const R* __restrict__ grid, long long nd, R* v);
template <>
MPM_D void load_node3<float>(const float* __restrict__ grid, long long nd, float* v)
{
    float4 q = __ldg(reinterpret_cast<const float4*>(grid) + nd);
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
}
template <>
MPM_D void load_node3<double>(const double* __restrict__ grid, long long nd, double* v)
{
    double2 a = __ldg(reinterpret_cast<const double2*>(grid) + 2 * nd);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = __ldg(grid + 4 * nd + 2);
}
template <typename R>
MPM_D void load_node4(const R* __restrict__ grid, long long nd, R* v);
template <>
MPM_D void load_node4<float>(const float* __restrict__ grid, long long nd, float* v)
{
    float4 q = __ldg(reinterpret_cast<const float4*>(grid) + nd);
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
}
template <>
MPM_D void load_node4<double>(const double* __restrict__ grid, long long nd, double* v)
{
    double2 a = __ldg(reinterpret_cast<const double2*>(grid) + 2 * nd);
    double2 b = __ldg(reinterpret_cast<const double2*>(grid) + 2 * nd + 1);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
}

// ------------------------------------------------------------------------
// Gather tile (FP32): the block's stencil bounding box of one or two node
// arrays (float4 per node) is copied into shared memory once, so the 64
// per-particle node reads hit shared memory instead of L1/L2.  Blocks whose
// box exceeds the budget read global memory directly.
// ------------------------------------------------------------------------
struct GTile {
    bool on;
    int b0, b1, b2, e1, e2;
    __device__ __forceinline__ int index(int i, int j, int k) const { return ((i - b0) * e1 + (j - b1)) * e2 + (k - b2); }
};

template <int K, int NA>
__device__ GTile stage_gather_tile(const KP<float>& kp, bool valid, const int* base, const float4* __restrict__ s0,
                                   const float4* __restrict__ s1, float4* d0, float4* d1, int cap)
{
    __shared__ int box[6];
    const int t = threadIdx.x, lane = t & 31;
    if (t < 3) box[t] = INT_MAX;
    else if (t < 6) box[t] = INT_MIN;
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int lo = __reduce_min_sync(0xffffffffu, valid ? base[a] : INT_MAX);
        const int hi = __reduce_max_sync(0xffffffffu, valid ? base[a] : INT_MIN);
        if (lane == 0) {
            atomicMin(&box[a], lo);
            atomicMax(&box[3 + a], hi);
        }
    }
    __syncthreads();
    GTile g;
    g.on = false;
    g.b0 = g.b1 = g.b2 = g.e1 = g.e2 = 0;
    if (cap > 0 && box[0] != INT_MAX) {
        const long long x0 = (long long)box[3] - box[0] + K, x1 = (long long)box[4] - box[1] + K,
                        x2 = (long long)box[5] - box[2] + K;
        if (x0 > 0 && x1 > 0 && x2 > 0 && x0 <= cap && x1 <= cap && x2 <= cap && x0 * x1 * x2 <= cap) {
            g.on = true;
            g.b0 = box[0];
            g.b1 = box[1];
            g.b2 = box[2];
            g.e1 = (int)x1;
            g.e2 = (int)x2;
            const int vol = (int)(x0 * x1 * x2);
            // u / e by a multiply-high: e >= K > 1 and u < 2^20 keep it exact
            const unsigned m2 = 0xFFFFFFFFu / (unsigned)g.e2 + 1u, m1 = 0xFFFFFFFFu / (unsigned)g.e1 + 1u;
            for (int u = t; u < vol; u += blockDim.x) {
                const int rr = (int)__umulhi((unsigned)u, m2), kk = u - rr * g.e2;
                const int ii = (int)__umulhi((unsigned)rr, m1), jj = rr - ii * g.e1;
                const int i = g.b0 + ii, j = g.b1 + jj, k = g.b2 + kk;
                float4 v0 = make_float4(0.f, 0.f, 0.f, 0.f), v1 = v0;
                if (in_grid(kp, i, j, k)) {
                    const long long nd = node_of(kp, i, j, k);
                    v0 = __ldg(s0 + nd);
                    if (NA == 2) v1 = __ldg(s1 + nd);
                }
                d0[u] = v0;
                if (NA == 2) d1[u] = v1;
            }
        }
    }
    __syncthreads();
    return g;
}

// ------------------------------------------------------------------ G2P

// G2P epilogue (ForwardSimulation.cpp:120-157): C from the gathered moments,
// J trust region, F update with smoothing, advection, stores of layer n+1.
template <typename R>
MPM_D void g2p_finish(const KP<R>& kp, long long ld, int p, const R* x, const R* F, const R* Ft, const R* vs,
                      const R* Cx, const R* Cy, const R* Cz, R* __restrict__ st1, R* __restrict__ trust,
                      R* x_out = nullptr, R* C_out = nullptr, R* F_out = nullptr)
{
    R Cn[9];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        Cn[r * 3 + 0] = kp.C0 * Cx[r];
        Cn[r * 3 + 1] = kp.C0 * Cy[r];
        Cn[r * 3 + 2] = kp.C0 * Cz[r];
    }
    // J trust region (ForwardSimulation.cpp:135-152)
    R s_tr = R(1);
    if (kp.jmin > R(0)) {
        R J0 = R(1) + det_minus_one(Ft);
        J0 = J0 > R(1e-6) ? J0 : R(1e-6);
        const R trC = Cn[0] + Cn[4] + Cn[8];
        if (trC < R(0)) {
            const R denom = kp.dt * trC;
            const R s = (kp.jmin / J0 - R(1)) / (denom < R(-1e-6) ? denom : R(-1e-6));
            if (s < R(1)) {
                s_tr = s < R(0) ? R(0) : s;
#pragma unroll
                for (int i = 0; i < 9; ++i) Cn[i] *= s_tr;
            }
        }
    }
    R IdtC[9], Fn[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) IdtC[i] = ((i % 4 == 0) ? R(1) : R(0)) + kp.dt * Cn[i];
    mul3(IdtC, Ft, Fn);
#pragma unroll
    for (int i = 0; i < 9; ++i) Fn[i] = Fn[i] * (R(1) - kp.s) + F[i] * kp.s;
    R x1[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) x1[a] = x[a] + kp.dt * vs[a];
    store_planes(st1 + ST_X * ld, ld, p, 3, x1);
    store_planes(st1 + ST_V * ld, ld, p, 3, vs);
    store_planes(st1 + ST_C * ld, ld, p, 9, Cn);
    store_planes(st1 + ST_F * ld, ld, p, 9, Fn);
    if (trust) trust[p] = s_tr;
    // the new state, for a caller that goes on with it (the fused G2P->P2G)
    if (x_out)
#pragma unroll
        for (int a = 0; a < 3; ++a) x_out[a] = x1[a];
    if (C_out)
#pragma unroll
        for (int i = 0; i < 9; ++i) C_out[i] = Cn[i];
    if (F_out)
#pragma unroll
        for (int i = 0; i < 9; ++i) F_out[i] = Fn[i];
}

// G2P gather: v = sum w v_i, Cacc[:,a] = sum w v_i dg_a, separable.
// CHECK = false for a particle whose whole stencil lies inside the grid (the
// common case): no per-node bounds checks, so every node load can issue
// without waiting on a predicate.
template <typename R, int K, bool CHECK>
MPM_D void g2p_gather(const KP<R>& kp, const Stencil<R, K>& sn, const R* __restrict__ grid, R* vs, R* Cx, R* Cy,
                      R* Cz)
{
    const long long sy = kp.dims[2], sx = (long long)kp.dims[1] * kp.dims[2];
    const long long base = ((long long)sn.base[0] * kp.dims[1] + sn.base[1]) * kp.dims[2] + sn.base[2];
#pragma unroll
    for (int a = 0; a < K; ++a) {
        const int i = sn.base[0] + a;
        if (CHECK && (unsigned)i >= (unsigned)kp.dims[0]) continue;
        R t0[3] = {0, 0, 0}, t1[3] = {0, 0, 0}, t2[3] = {0, 0, 0};
#pragma unroll
        for (int b = 0; b < K; ++b) {
            const int j = sn.base[1] + b;
            if (CHECK && (unsigned)j >= (unsigned)kp.dims[1]) continue;
            R s0[3] = {0, 0, 0}, s2[3] = {0, 0, 0};
            const long long row = base + a * sx + b * sy;
#pragma unroll
            for (int c = 0; c < K; ++c) {
                const int k = sn.base[2] + c;
                if (CHECK && (unsigned)k >= (unsigned)kp.dims[2]) continue;
                R vi[3];
                load_node3(grid, row + c, vi);
                const R wz = sn.w[2][c], wzg = wz * sn.g[2][c];
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    s0[r] += wz * vi[r];
                    s2[r] += wzg * vi[r];
                }
            }
            const R wy = sn.w[1][b], wyg = wy * sn.g[1][b];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                t0[r] += wy * s0[r];
                t1[r] += wyg * s0[r];
                t2[r] += wy * s2[r];
            }
        }
        const R wx = sn.w[0][a], wxg = wx * sn.g[0][a];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            vs[r] += wx * t0[r];
            Cx[r] += wxg * t0[r];
            Cy[r] += wx * t1[r];
            Cz[r] += wx * t2[r];
        }
    }
}

template <typename R, int K>
MPM_D bool stencil_inside(const KP<R>& kp, const Stencil<R, K>& sn)
{
    bool in = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) in &= sn.base[a] >= 0 && sn.base[a] + K <= kp.dims[a];
    return in;
}

template <typename R, int K>
__global__ void __launch_bounds__(kThreads, MPM_G2P_MIN_BLOCKS) k_g2p(KP<R> kp, int n, long long ld, const R* __restrict__ st,
                                                   const R* __restrict__ dfc, const R* __restrict__ grid,
                                                   R* __restrict__ st1, R* __restrict__ trust)
{
    long long goff;
    bind_instance(kp, n, goff);
    grid += goff * 4;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    R x[3], F[9], Ft[9];
    load_planes(st + ST_X * ld, ld, p, 3, x);
    load_Ft(st, dfc, ld, p, F, Ft);
    Stencil<R, K> sn;
    make_stencil<R, K>(x, kp.gmin, kp.dx, kp.inv_dx, sn, false);
    R vs[3] = {0, 0, 0}, Cx[3] = {0, 0, 0}, Cy[3] = {0, 0, 0}, Cz[3] = {0, 0, 0};
    // (the plain FP64 form keeps one checked path)
    if (sizeof(R) == 4 && stencil_inside(kp, sn)) g2p_gather<R, K, false>(kp, sn, grid, vs, Cx, Cy, Cz);
    else g2p_gather<R, K, true>(kp, sn, grid, vs, Cx, Cy, Cz);
    g2p_finish(kp, ld, p, x, F, Ft, vs, Cx, Cy, Cz, st1, trust);
}

// ------------------------------------------------------------- adjoint

// P_op_2^T for one particle (BackPropagation.cpp:22-32): dL/dv_next, dL/dC_next
// and the part of dL/dFt that does not pass through the grid.  In exact mode
// the trust-region scale of the step is differentiated as well.
template <typename R>
struct PostAdj {
    R vbar[3], Cbar[9], Fpart[9];
};

template <typename R>
MPM_D void post_adjoint(const KP<R>& kp, long long ld, int p, const R* Ft, const R* __restrict__ st1,
                        const R* __restrict__ g1, const R* __restrict__ trust, PostAdj<R>& o)
{
    R C1[9], gF1[9], gx1[3], gv1[3], gC1[9];
    load_planes(st1 + ST_C * ld, ld, p, 9, C1);
    load_planes(g1 + ST_F * ld, ld, p, 9, gF1);
    load_planes(g1 + ST_X * ld, ld, p, 3, gx1);
    load_planes(g1 + ST_V * ld, ld, p, 3, gv1);
    load_planes(g1 + ST_C * ld, ld, p, 9, gC1);
    R IdtC[9], t[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) IdtC[i] = ((i % 4 == 0) ? R(1) : R(0)) + kp.dt * C1[i];
    mulTN3(IdtC, gF1, t);  // (I + dt C1)^T g
#pragma unroll
    for (int a = 0; a < 3; ++a) o.vbar[a] = kp.dt * gx1[a] + gv1[a];
    R gFtT[9];
    mulNT3(gF1, Ft, gFtT);  // g Ft^T
    const R cf = kp.exact ? (R(1) - kp.s) * kp.dt : kp.dt;
#pragma unroll
    for (int i = 0; i < 9; ++i) o.Cbar[i] = cf * gFtT[i] + gC1[i];
    if (kp.exact) {
#pragma unroll
        for (int i = 0; i < 9; ++i) o.Fpart[i] = (R(1) - kp.s) * t[i];
        if (kp.jmin > R(0) && trust) {
            const R s_tr = trust[p];
            if (s_tr <= R(0)) {
#pragma unroll
                for (int i = 0; i < 9; ++i) o.Cbar[i] = R(0);
            } else if (s_tr < R(1)) {
                R Cp[9];
#pragma unroll
                for (int i = 0; i < 9; ++i) Cp[i] = C1[i] / s_tr;
                const R trCp = Cp[0] + Cp[4] + Cp[8];
                const R denom = kp.dt * trCp;
                const R q = dot9(o.Cbar, Cp);
                const R dsdtr = denom < R(-1e-6) ? -s_tr / trCp : R(0);
                R c[9];
                cof3(Ft, c);
                const R J0 = R(1) + det_minus_one(Ft);
                const R dsdJ0 = J0 > R(1e-6) ? -kp.jmin / (J0 * J0 * (denom < R(-1e-6) ? denom : R(-1e-6))) : R(0);
#pragma unroll
                for (int i = 0; i < 9; ++i) {
                    o.Cbar[i] = s_tr * o.Cbar[i] + ((i % 4 == 0) ? q * dsdtr : R(0));
                    o.Fpart[i] += q * dsdJ0 * c[i];  // J0 Ft^{-T} = cof(Ft)
                }
            }
        }
    } else {
        // reference: (1-s)(I+dtC1)^T g + s g, plus the second (I+dtC1)^T g
        // that BackPropagation.cpp:140 adds
#pragma unroll
        for (int i = 0; i < 9; ++i) o.Fpart[i] = (R(2) - kp.s) * t[i] + kp.s * gF1[i];
    }
}

template <typename R, int K>
__global__ void __launch_bounds__(kThreads) k_g2p_adj(KP<R> kp, int n, long long ld, const R* __restrict__ st,
                                                       const R* __restrict__ dfc, const R* __restrict__ st1,
                                                       const R* __restrict__ g1, const R* __restrict__ trust,
                                                       R* __restrict__ adj, int tile_cap)
{
    extern __shared__ __align__(16) unsigned char smem[];
    long long goff;
    bind_instance(kp, n, goff);
    adj += goff * 4;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < n;
    Stencil<R, K> sten;
    R vb[3], CC[9];
    if (valid) {
        R x[3], F[9], Ft[9];
        load_planes(st + ST_X * ld, ld, p, 3, x);
        load_Ft(st, dfc, ld, p, F, Ft);
        PostAdj<R> o;
        post_adjoint(kp, ld, p, Ft, st1, g1, trust, o);
#pragma unroll
        for (int a = 0; a < 3; ++a) vb[a] = o.vbar[a];
#pragma unroll
        for (int i = 0; i < 9; ++i) CC[i] = kp.C0 * o.Cbar[i];
        make_stencil<R, K>(x, kp.gmin, kp.dx, kp.inv_dx, sten, false);
    }
    Scatter<R, K, 3> sc;
    sc.setup(valid, sten.base, smem, tile_cap);
    if (valid) {
        walk_rotated<R, K>(sten, [&](int i, int j, int k, R w, R gx, R gy, R gz) {
            R val[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) val[r] = w * (vb[r] + CC[r * 3] * gx + CC[r * 3 + 1] * gy + CC[r * 3 + 2] * gz);
            sc.add(kp, adj, i, j, k, val);
        });
    }
    sc.flush(kp, adj);
}

// P_op_1 + P2G with the segmented scatter (FP32 path); DET: fixed-point sums
template <int K, bool DET>
__global__ void __launch_bounds__(kThreads, MPM_P2G_MIN_BLOCKS) k_p2g_seg(KP<float> kp, int n, long long ld, const float* __restrict__ st,
                                                       const float* __restrict__ dfc, const float* __restrict__ co,
                                                       float* __restrict__ grid, int tile_cap, FixArgs fx)
{
    extern __shared__ __align__(16) unsigned char smem[];
    long long goff;
    bind_instance(kp, n, goff);
    if constexpr (DET) fx.acc += goff * 4;
    else grid += goff * 4;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < n;
    Stencil<float, K> sten;
    float A[9], mv[3], mass = 0.f;
    if (valid) {
        float x[3], v[3], C[9], F[9], Ft[9];
        load_planes(st + ST_X * ld, ld, p, 3, x);
        load_planes(st + ST_V * ld, ld, p, 3, v);
        load_planes(st + ST_C * ld, ld, p, 9, C);
        load_Ft(st, dfc, ld, p, F, Ft);
        mass = co[CO_M * ld + p];
        const float vol = co[CO_VOL * ld + p], lam = co[CO_LAM * ld + p], mu = co[CO_MU * ld + p];
        float PF[9];
        stress_pf(kp.material, Ft, lam, mu, PF);
        const float trC = C[0] + C[4] + C[8];
        const float k1 = -kp.C0 * kp.dt * vol;
#pragma unroll
        for (int i = 0; i < 9; ++i) A[i] = k1 * (PF[i] + ((i % 4 == 0) ? kp.bulk * trC : 0.f)) + mass * C[i];
#pragma unroll
        for (int a = 0; a < 3; ++a) mv[a] = mass * v[a] * kp.dragf;
        make_stencil<float, K>(x, kp.gmin, kp.dx, kp.inv_dx, sten, false);
    }
    if constexpr (DET) {
        const float bm = fix_mass_bound(fx);
        const float sp = pow2f(fix_exponent(bm * fx.speed)), sm = pow2f(fix_exponent(bm));
        const float scale[4] = {sp, sp, sp, sm};
        seg_scatter<K, 4, true>(kp, valid, sten, mv, mass, A, grid, tile_cap, smem, &fx, scale);
    } else {
        seg_scatter<K, 4>(kp, valid, sten, mv, mass, A, grid, tile_cap, smem);
    }
}

// G2P of step i fused with P2G of step i+1 (FP32, segmented scatter).  The
// state G2P forms for layer i+1 -- stored as usual for the tape -- stays in
// registers and feeds the next step's stress and scatter, so that step does
// not read it back; layer i+1 has no control (a forward pass zeroes the
// control of every layer it writes, ForwardSimulation.cpp:155).  grid is
// step i's updated grid (read); grid1 is step i+1's, zeroed (scattered into).
template <int K>
__global__ void __launch_bounds__(kThreads, MPM_G2P2G_MIN_BLOCKS)
k_g2p2g(KP<float> kp, int n, long long ld, const float* __restrict__ st, const float* __restrict__ dfc,
        const float* __restrict__ co, const float* __restrict__ grid, float* __restrict__ st1,
        float* __restrict__ trust, float* __restrict__ grid1, int tile_cap)
{
    extern __shared__ __align__(16) unsigned char smem[];
    long long goff;
    bind_instance(kp, n, goff);
    grid += goff * 4;
    grid1 += goff * 4;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < n;
    Stencil<float, K> sten;
    float A[9], mv[3], mass = 0.f;
    if (valid) {
        float x1[3], vs[3] = {0.f, 0.f, 0.f}, C1[9], F1[9];
        {
            float x[3], F[9], Ft[9];
            load_planes(st + ST_X * ld, ld, p, 3, x);
            load_Ft(st, dfc, ld, p, F, Ft);
            Stencil<float, K> sn;
            make_stencil<float, K>(x, kp.gmin, kp.dx, kp.inv_dx, sn, false);
            float Cx[3] = {0, 0, 0}, Cy[3] = {0, 0, 0}, Cz[3] = {0, 0, 0};
            if (stencil_inside(kp, sn)) g2p_gather<float, K, false>(kp, sn, grid, vs, Cx, Cy, Cz);
            else g2p_gather<float, K, true>(kp, sn, grid, vs, Cx, Cy, Cz);
            g2p_finish(kp, ld, p, x, F, Ft, vs, Cx, Cy, Cz, st1, trust, x1, C1, F1);
        }
        mass = co[CO_M * ld + p];
        const float vol = co[CO_VOL * ld + p], lam = co[CO_LAM * ld + p], mu = co[CO_MU * ld + p];
        float PF[9];
        stress_pf(kp.material, F1, lam, mu, PF);
        const float trC = C1[0] + C1[4] + C1[8];
        const float k1 = -kp.C0 * kp.dt * vol;
#pragma unroll
        for (int i = 0; i < 9; ++i) A[i] = k1 * (PF[i] + ((i % 4 == 0) ? kp.bulk * trC : 0.f)) + mass * C1[i];
#pragma unroll
        for (int a = 0; a < 3; ++a) mv[a] = mass * vs[a] * kp.dragf;
        make_stencil<float, K>(x1, kp.gmin, kp.dx, kp.inv_dx, sten, false);
    }
    seg_scatter<K, 4>(kp, valid, sten, mv, mass, A, grid1, tile_cap, smem);
}

// Deterministic mode: the node sums of P2G (fixed point) -> mass clamp +
// G_op, as k_grid_update; clears the accumulators for the next step
__global__ void k_grid_update_fix(KP<float> kp, long long nn, FixArgs fx, float* __restrict__ grid)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    const float bm = fix_mass_bound(fx);
    const float ip = pow2f(-fix_exponent(bm * fx.speed)), im = pow2f(-fix_exponent(bm));
    longlong2* a = reinterpret_cast<longlong2*>(fx.acc + 4 * i);
    const longlong2 q01 = a[0], q23 = a[1];
    if ((q01.x | q01.y | q23.x | q23.y) != 0) {  // most nodes are empty: leave their zeros
        a[0] = make_longlong2(0, 0);
        a[1] = make_longlong2(0, 0);
    }
    const long long lim = 1ll << 62;
    if (q01.x >= lim || q01.x <= -lim || q01.y >= lim || q01.y <= -lim || q23.x >= lim || q23.x <= -lim ||
        q23.y >= lim || q23.y <= -lim || (fx.ctl[3] & 1u)) {
        // out of the fixed-point range (or a non-finite contribution this
        // pass): the step's result is non-finite, as an overflowing float sum
        // would make it
        atomicOr(&fx.ctl[3], 2u);
        reinterpret_cast<float4*>(grid)[i] = make_float4(NAN, NAN, NAN, NAN);
        return;
    }
    float m = __ll2float_rn(q23.y) * im;
    if (m < 0.f) m = 0.f;
    float v0 = 0.f, v1 = 0.f, v2 = 0.f;
    if (m > 1e-12f) {
        v0 = __ll2float_rn(q01.x) * ip / m + kp.dtf[0];
        v1 = __ll2float_rn(q01.y) * ip / m + kp.dtf[1];
        v2 = __ll2float_rn(q23.x) * ip / m + kp.dtf[2];
    }
    reinterpret_cast<float4*>(grid)[i] = make_float4(v0, v1, v2, m);
}

// largest particle mass -> fix_ctl[0] (bits of a non-negative float order
// like the floats)
__global__ void k_fix_mass_max(int n, long long ld, const float* __restrict__ co, unsigned* ctl)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const float m = p < n ? fabsf(co[CO_M * ld + p]) : 0.f;
    const unsigned b = __reduce_max_sync(0xffffffffu, __float_as_uint(m == m ? m : 0.f));
    if ((threadIdx.x & 31) == 0 && b) atomicMax(&ctl[0], b);
}

// P_op_2^T + G2P^T with the segmented scatter (FP32 path)
template <int K>
__global__ void __launch_bounds__(kThreads) k_g2p_adj_seg(KP<float> kp, int n, long long ld,
                                                           const float* __restrict__ st, const float* __restrict__ dfc,
                                                           const float* __restrict__ st1, const float* __restrict__ g1,
                                                           const float* __restrict__ trust, float* __restrict__ adj,
                                                           int tile_cap)
{
    extern __shared__ __align__(16) unsigned char smem[];
    long long goff;
    bind_instance(kp, n, goff);
    adj += goff * 4;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < n;
    Stencil<float, K> sten;
    float vb[3], CC[9];
    if (valid) {
        float x[3], F[9], Ft[9];
        load_planes(st + ST_X * ld, ld, p, 3, x);
        load_Ft(st, dfc, ld, p, F, Ft);
        PostAdj<float> o;
        post_adjoint(kp, ld, p, Ft, st1, g1, trust, o);
#pragma unroll
        for (int a = 0; a < 3; ++a) vb[a] = o.vbar[a];
#pragma unroll
        for (int i = 0; i < 9; ++i) CC[i] = kp.C0 * o.Cbar[i];
        make_stencil<float, K>(x, kp.gmin, kp.dx, kp.inv_dx, sten, false);
    }
    seg_scatter<K, 3>(kp, valid, sten, vb, 0.f, CC, adj, tile_cap, smem);
}

// Deterministic mode, first half of P_op_2^T + G2P^T: the scatter inputs
// (dL/dv_next, C0 dL/dC_next) of every particle into 12 scratch planes and
// their largest magnitudes into fix_ctl[1], fix_ctl[2] (they set the
// fixed-point scale of the scatter)
template <int K>
__global__ void __launch_bounds__(kThreads) k_g2p_adj_prep(KP<float> kp, int n, long long ld,
                                                            const float* __restrict__ st, const float* __restrict__ dfc,
                                                            const float* __restrict__ st1, const float* __restrict__ g1,
                                                            const float* __restrict__ trust, FixArgs fx,
                                                            float* __restrict__ scr)
{
    long long goff;
    bind_instance(kp, n, goff);
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    float vmx = 0.f, cmx = 0.f;
    if (p < n) {
        float F[9], Ft[9];
        load_Ft(st, dfc, ld, p, F, Ft);
        PostAdj<float> o;
        post_adjoint(kp, ld, p, Ft, st1, g1, trust, o);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            scr[(long long)a * ld + p] = o.vbar[a];
            vmx = fmaxf(vmx, fabsf(o.vbar[a]));
        }
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const float c = kp.C0 * o.Cbar[i];
            scr[(long long)(3 + i) * ld + p] = c;
            cmx = fmaxf(cmx, fabsf(c));
        }
    }
    const unsigned a = __reduce_max_sync(0xffffffffu, __float_as_uint(vmx));
    const unsigned b = __reduce_max_sync(0xffffffffu, __float_as_uint(cmx));
    if ((threadIdx.x & 31) == 0) {
        if (a) atomicMax(&fx.ctl[1], a);
        if (b) atomicMax(&fx.ctl[2], b);
    }
}

// Deterministic mode, second half: the G2P^T scatter in fixed point
template <int K>
__global__ void __launch_bounds__(kThreads) k_g2p_adj_fix(KP<float> kp, int n, long long ld,
                                                           const float* __restrict__ st, const float* __restrict__ scr,
                                                           FixArgs fx, int tile_cap)
{
    extern __shared__ __align__(16) unsigned char smem[];
    long long goff;
    bind_instance(kp, n, goff);
    fx.acc += goff * 4;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < n;
    Stencil<float, K> sten;
    float vb[3], CC[9];
    if (valid) {
        float x[3];
        load_planes(st + ST_X * ld, ld, p, 3, x);
        load_planes(scr, ld, p, 3, vb);
        load_planes(scr + 3 * ld, ld, p, 9, CC);
        make_stencil<float, K>(x, kp.gmin, kp.dx, kp.inv_dx, sten, false);
    }
    const float sa = pow2f(fix_exponent(fix_adj_bound(fx)));
    const float scale[3] = {sa, sa, sa};
    seg_scatter<K, 3, true>(kp, valid, sten, vb, 0.f, CC, nullptr, tile_cap, smem, &fx, scale);
}

// G_op^T (BackPropagation.cpp:59-72) reading the fixed-point dL/dv sums;
// writes all four adjoint slots and clears the accumulators
__global__ void k_grid_adj_fix(KP<float> kp, long long nn, const float* __restrict__ grid, FixArgs fx,
                               float* __restrict__ adj)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    const float inv = pow2f(-fix_exponent(fix_adj_bound(fx)));
    longlong2* a = reinterpret_cast<longlong2*>(fx.acc + 4 * i);
    const longlong2 q01 = a[0], q23 = a[1];
    if ((q01.x | q01.y | q23.x | q23.y) != 0) {
        a[0] = make_longlong2(0, 0);
        a[1] = make_longlong2(0, 0);
    }
    const long long lim = 1ll << 62;
    if (q01.x >= lim || q01.x <= -lim || q01.y >= lim || q01.y <= -lim || q23.x >= lim || q23.x <= -lim ||
        (fx.ctl[3] & 1u)) {
        atomicOr(&fx.ctl[3], 2u);
        reinterpret_cast<float4*>(adj)[i] = make_float4(NAN, NAN, NAN, NAN);
        return;
    }
    const float d0 = __ll2float_rn(q01.x) * inv, d1 = __ll2float_rn(q01.y) * inv, d2 = __ll2float_rn(q23.x) * inv;
    const float4 g = reinterpret_cast<const float4*>(grid)[i];
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (fabsf(g.w) > 1e-12f) {
        float v0 = g.x, v1 = g.y, v2 = g.z;
        if (kp.exact) {
            v0 -= kp.dtf[0];
            v1 -= kp.dtf[1];
            v2 -= kp.dtf[2];
        }
        const float im = 1.f / g.w;
        out = make_float4(d0 * im, d1 * im, d2 * im, -(v0 * d0 + v1 * d1 + v2 * d2) * im);
    }
    reinterpret_cast<float4*>(adj)[i] = out;
}

// G_op^T (BackPropagation.cpp:59-72)
template <typename R>
__global__ void k_grid_adj(KP<R> kp, long long nn, const R* __restrict__ grid, R* __restrict__ adj,
                           R* __restrict__ zero_next)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    if (zero_next) {  // the adjoint grid of the next (earlier) step
        if constexpr (sizeof(R) == 4) reinterpret_cast<float4*>(zero_next)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        else {
            R* z = zero_next + 4 * i;
            z[0] = z[1] = z[2] = z[3] = R(0);
        }
    }
    if constexpr (sizeof(R) == 4) {
        // 16-byte accesses; a massless node's adjoint is zeroed unread
        const float4 q = __ldg(reinterpret_cast<const float4*>(grid) + i);
        float4* dp = reinterpret_cast<float4*>(adj) + i;
        if (fabsf(q.w) > 1e-12f) {
            const float4 dd = *dp;
            float v0 = q.x, v1 = q.y, v2 = q.z;
            if (kp.exact) {
                v0 -= kp.dtf[0];
                v1 -= kp.dtf[1];
                v2 -= kp.dtf[2];
            }
            const float im = 1.f / q.w;
            *dp = make_float4(dd.x * im, dd.y * im, dd.z * im, -(v0 * dd.x + v1 * dd.y + v2 * dd.z) * im);
        } else {
            *dp = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        return;
    }
    const R* g = grid + 4 * i;
    R* d = adj + 4 * i;
    const R m = g[3];
    if (fabs(m) > R(1e-12)) {
        R v0 = g[0], v1 = g[1], v2 = g[2];
        if (kp.exact) {
            v0 -= kp.dtf[0];
            v1 -= kp.dtf[1];
            v2 -= kp.dtf[2];
        }
        const R d0 = d[0], d1 = d[1], d2 = d[2];
        const R im = R(1) / m;
        d[3] = -(v0 * d0 + v1 * d1 + v2 * d2) * im;
        d[0] = d0 * im;
        d[1] = d1 * im;
        d[2] = d2 * im;
    } else {
        d[0] = d[1] = d[2] = d[3] = R(0);
    }
}

// The P2G-transpose gather (FP32 tile or global reads).  TILE: every node
// of the block's stencils is in the staged tile, which holds zeros outside
// the grid, so the per-node grid bounds checks are not needed.
template <typename R, int K, bool TILE>
MPM_D void p2g_adj_gather(const KP<R>& kp, const Stencil<R, K>& sn, const GTile& tl, const float4* ta, const float4* tg,
                          const R* __restrict__ adj, const R* __restrict__ grid, R mass, const R* mvv, const R* A,
                          const R* vbar, const R* CC, R* M1, R* ax, R* bp, R* bv)
{
    // Separable accumulation over the K^3 stencil.  Per node n = (a,b,c) with
    // d = (dL/dp, dL/dm) and v_i the node velocity:
    //   sig_n = m dL/dm + (m v' + A dg).dL/dp + v_i.(vbar + C0 Cbar dg)
    //   ax += sig_n grad w_n,  bp += w_n dL/dp,  bv += w_n v_i,
    //   M1 += w_n dL/dp dg^T
    // with w_n = wx_a wy_b wz_c and grad w_n = -(1/dx)(sx wy wz, wx sy wz,
    // wx wy sz); the sums over c, then b, are folded into per-(a,b) and
    // per-a partials so each node costs ~24 FMAs.
#pragma unroll
    for (int a = 0; a < K; ++a) {
        const int i = sn.base[0] + a;
        if (!TILE && (unsigned)i >= (unsigned)kp.dims[0]) continue;
        const R gxa = sn.g[0][a];
        R Pa[3], Qa[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            Pa[r] = mvv[r] + A[r * 3] * gxa;
            Qa[r] = vbar[r] + CC[r * 3] * gxa;
        }
        R Tw[3] = {0, 0, 0}, Tv[3] = {0, 0, 0}, Tgy[3] = {0, 0, 0}, Tgz[3] = {0, 0, 0};
        R Sww = 0, Ssw = 0, Sws = 0;
#pragma unroll
        for (int b = 0; b < K; ++b) {
            const int j = sn.base[1] + b;
            if (!TILE && (unsigned)j >= (unsigned)kp.dims[1]) continue;
            const R gyb = sn.g[1][b];
            R Pab[3], Qab[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                Pab[r] = Pa[r] + A[r * 3 + 1] * gyb;
                Qab[r] = Qa[r] + CC[r * 3 + 1] * gyb;
            }
            R U[3] = {0, 0, 0}, UV[3] = {0, 0, 0}, Ug[3] = {0, 0, 0};
            R Vw = 0, Vs = 0;
            const long long row = TILE ? 0 : ((long long)i * kp.dims[1] + j) * kp.dims[2];
            const int trow = TILE ? tl.index(i, j, 0) : 0;  // + k gives index(i, j, k)
#pragma unroll
            for (int c = 0; c < K; ++c) {
                const int k = sn.base[2] + c;
                if (!TILE && (unsigned)k >= (unsigned)kp.dims[2]) continue;
                R d[4], vi[3];
                if constexpr (TILE) {
                    const float4 qa = ta[trow + k], qg = tg[trow + k];
                    d[0] = (R)qa.x;
                    d[1] = (R)qa.y;
                    d[2] = (R)qa.z;
                    d[3] = (R)qa.w;
                    vi[0] = (R)qg.x;
                    vi[1] = (R)qg.y;
                    vi[2] = (R)qg.z;
                } else {
                    load_node4(adj, row + k, d);
                    load_node3(grid, row + k, vi);
                }
                const R gzc = sn.g[2][c], wc = sn.w[2][c];
                R sig = mass * d[3];
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    sig += (Pab[r] + A[r * 3 + 2] * gzc) * d[r];
                    sig += vi[r] * (Qab[r] + CC[r * 3 + 2] * gzc);
                }
                const R wcg = wc * gzc;
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    U[r] += wc * d[r];
                    UV[r] += wc * vi[r];
                    Ug[r] += wcg * d[r];
                }
                Vw += wc * sig;
                Vs += sn.s[2][c] * sig;
            }
            const R wb = sn.w[1][b], wbg = wb * gyb;
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                Tw[r] += wb * U[r];
                Tv[r] += wb * UV[r];
                Tgy[r] += wbg * U[r];
                Tgz[r] += wb * Ug[r];
            }
            Sww += wb * Vw;
            Ssw += sn.s[1][b] * Vw;
            Sws += wb * Vs;
        }
        const R wa = sn.w[0][a], wag = wa * gxa;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            bp[r] += wa * Tw[r];
            bv[r] += wa * Tv[r];
            M1[r * 3 + 0] += wag * Tw[r];
            M1[r * 3 + 1] += wa * Tgy[r];
            M1[r * 3 + 2] += wa * Tgz[r];
        }
        ax[0] += sn.s[0][a] * Sww;
        ax[1] += wa * Ssw;
        ax[2] += wa * Sws;
    }
}

// P2G^T + P_op_1^T (BackPropagation.cpp:76-143)
template <typename R, int K>
__global__ void __launch_bounds__(kThreads, MPM_P2G_ADJ_MIN_BLOCKS) k_p2g_adj(KP<R> kp, int n, long long ld, const R* __restrict__ st,
                                                       const R* __restrict__ dfc, const R* __restrict__ co,
                                                       const R* __restrict__ st1, const R* __restrict__ g1,
                                                       const R* __restrict__ trust, const R* __restrict__ grid,
                                                       const R* __restrict__ adj, R* __restrict__ g,
                                                       R* __restrict__ gFt_out, R* __restrict__ glam,
                                                       R* __restrict__ gmu, int cap)
{
    extern __shared__ __align__(16) unsigned char smem[];
    long long goff;
    bind_instance(kp, n, goff);
    grid += goff * 4;
    adj += goff * 4;
    // tail threads of the block mirror particle n-1 (never stored) so the
    // whole block can take part in staging the node tile
    const int p_raw = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p_raw < n;
    const int p = valid ? p_raw : n - 1;
    R x[3], v[3], C[9], F[9], Ft[9];
    load_planes(st + ST_X * ld, ld, p, 3, x);
    load_planes(st + ST_V * ld, ld, p, 3, v);
    load_planes(st + ST_C * ld, ld, p, 9, C);
    load_Ft(st, dfc, ld, p, F, Ft);
    const R mass = co[CO_M * ld + p], vol = co[CO_VOL * ld + p], lam = co[CO_LAM * ld + p], mu = co[CO_MU * ld + p];
    // running Lame gradient sums, read here so that the read is not the
    // last dependency of the block
    const R glam0 = glam ? glam[p] : R(0), gmu0 = gmu ? gmu[p] : R(0);
    Inv<R> iv;
    invariants(Ft, iv);
    R P[9], Rm[9], S[9], PF[9], A[9];
    pk(kp.material, Ft, lam, mu, iv, P, Rm, S);
    mulNT3(P, Ft, PF);
    const R trC = C[0] + C[4] + C[8];
    const R k1 = -kp.C0 * kp.dt * vol;
#pragma unroll
    for (int i = 0; i < 9; ++i) A[i] = k1 * (PF[i] + ((i % 4 == 0) ? kp.bulk * trC : R(0))) + mass * C[i];
    R mvv[3];
    const R mf = kp.exact ? kp.dragf : R(1);
#pragma unroll
    for (int a = 0; a < 3; ++a) mvv[a] = mass * v[a] * mf;
    PostAdj<R> o;
    post_adjoint(kp, ld, p, Ft, st1, g1, trust, o);
    R CC[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) CC[i] = kp.C0 * o.Cbar[i];

    Stencil<R, K> sn;
    make_stencil<R, K>(x, kp.gmin, kp.dx, kp.inv_dx, sn, true);
    GTile tl;
    tl.on = false;
    tl.b0 = tl.b1 = tl.b2 = tl.e1 = tl.e2 = 0;
    float4* ta = reinterpret_cast<float4*>(smem);
    float4* tg = ta + (cap > 0 ? cap : 0);
    if constexpr (sizeof(R) == 4) {
        tl = stage_gather_tile<K, 2>(kp, true, sn.base, reinterpret_cast<const float4*>(adj),
                                     reinterpret_cast<const float4*>(grid), ta, tg, cap);
    }
    R M1[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, ax[3] = {0, 0, 0}, bp[3] = {0, 0, 0}, bv[3] = {0, 0, 0};
    if constexpr (sizeof(R) == 4) {
        if (tl.on)
            p2g_adj_gather<R, K, true>(kp, sn, tl, ta, tg, adj, grid, mass, mvv, A, o.vbar, CC, M1, ax, bp, bv);
        else
            p2g_adj_gather<R, K, false>(kp, sn, tl, ta, tg, adj, grid, mass, mvv, A, o.vbar, CC, M1, ax, bp, bv);
    } else {
        p2g_adj_gather<R, K, false>(kp, sn, tl, ta, tg, adj, grid, mass, mvv, A, o.vbar, CC, M1, ax, bp, bv);
    }
    {
        const R nidx = -kp.inv_dx;
        ax[0] *= nidx;
        ax[1] *= nidx;
        ax[2] *= nidx;
    }
    if (!valid) return;
    R gx1[3];
    load_planes(g1 + ST_X * ld, ld, p, 3, gx1);
    R gx[3], gv[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const R AtB = A[r] * bp[0] + A[3 + r] * bp[1] + A[6 + r] * bp[2];
        const R CtV = CC[r] * bv[0] + CC[3 + r] * bv[1] + CC[6 + r] * bv[2];
        gx[r] = ax[r] - AtB - CtV + gx1[r];
        gv[r] = mass * kp.dragf * bp[r];
    }
    R gC[9];
    const R kb = k1 * kp.bulk;
    const R trM = M1[0] + M1[4] + M1[8];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        R add = R(0);
        if (i % 4 == 0) add = kp.exact ? kb * trM : kb * M1[i];
        gC[i] = mass * M1[i] + add;
    }
    R t1[9], t2[9], gP[9], hv[9], gF[9];
    mul3(M1, Ft, t1);
    mulTN3(M1, P, t2);
#pragma unroll
    for (int i = 0; i < 9; ++i) gP[i] = k1 * t1[i];
    pk_vjp(kp.material, kp.exact != 0, Ft, lam, mu, iv, Rm, S, gP, hv);
#pragma unroll
    for (int i = 0; i < 9; ++i) gF[i] = o.Fpart[i] + k1 * t2[i] + hv[i];
    if (gFt_out) store_planes(gFt_out, ld, p, 9, gF);
    if (kp.exact) {
        R gF1[9];
        load_planes(g1 + ST_F * ld, ld, p, 9, gF1);
#pragma unroll
        for (int i = 0; i < 9; ++i) gF[i] += kp.s * gF1[i];
    }
    store_planes(g + ST_X * ld, ld, p, 3, gx);
    store_planes(g + ST_V * ld, ld, p, 3, gv);
    store_planes(g + ST_F * ld, ld, p, 9, gF);
    store_planes(g + ST_C * ld, ld, p, 9, gC);
    if (glam || gmu) {
        R dm = 0, dl = 0;
        if (kp.material == MAT_FCR) {
            const R kk = iv.Jm1c * iv.Jc;
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                dm += gP[i] * R(2) * (Ft[i] - Rm[i]);
                dl += gP[i] * kk * iv.Fit[i];
            }
        } else {
            const R lj = log(iv.Jc);
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                dm += gP[i] * (Ft[i] - iv.Fit[i]);
                dl += gP[i] * lj * iv.Fit[i];
            }
        }
        if (gmu) gmu[p] = gmu0 + dm;
        if (glam) glam[p] = glam0 + dl;
    }
}

// ---------------------------------------------------------------- loss

template <typename R>
MPM_D double block_sum(double v, double* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    }
    __syncthreads();
    return s;  // valid in thread 0
}

template <typename R, int K>
__global__ void __launch_bounds__(kThreads) k_mass_p2g(KP<R> kp, int n, long long ld, const R* __restrict__ st,
                                                        const R* __restrict__ co, R* __restrict__ gm)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    R x[3];
    load_planes(st + ST_X * ld, ld, p, 3, x);
    const R m = co[CO_M * ld + p];
    Stencil<R, K> sn;
    make_stencil<R, K>(x, kp.gmin, kp.dx, kp.inv_dx, sn, false);
    walk_rotated<R, K>(sn, [&](int i, int j, int k, R w, R, R, R) {
        if (in_grid(kp, i, j, k)) atomicAdd(&gm[node_of(kp, i, j, k)], w * m);
    });
}

// deterministic mode: the loss's mass P2G into the fixed-point slot 3
template <int K>
__global__ void __launch_bounds__(kThreads) k_mass_p2g_fix(KP<float> kp, int n, long long ld,
                                                            const float* __restrict__ st, const float* __restrict__ co,
                                                            FixArgs fx)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float x[3];
    load_planes(st + ST_X * ld, ld, p, 3, x);
    const float m = co[CO_M * ld + p];
    const float scale = pow2f(fix_exponent(fix_mass_bound(fx)));
    Stencil<float, K> sn;
    make_stencil<float, K>(x, kp.gmin, kp.dx, kp.inv_dx, sn, false);
    bool ovf = false;
    walk_rotated<float, K>(sn, [&](int i, int j, int k, float w, float, float, float) {
        if (in_grid(kp, i, j, k)) atomicAdd(&fx.acc[node_of(kp, i, j, k) * 4 + 3], to_fix(w * m, scale, ovf));
    });
    if (ovf) atomicOr(&fx.ctl[3], 1u);
}

__global__ void k_fix_mass_out(long long nn, FixArgs fx, float* __restrict__ gm)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    const long long q = (long long)fx.acc[4 * i + 3];
    if (q) fx.acc[4 * i + 3] = 0ull;
    gm[i] = (fx.ctl[3] & 1u) ? NAN : __ll2float_rn(q) * pow2f(-fix_exponent(fix_mass_bound(fx)));
}

// Deterministic reductions: each block writes its partial sum(s) to
// parts[block * stride + column]; k_sum_parts adds them up in a fixed order
// (one warp per column, lane-strided, then a fixed shuffle tree).
__global__ void k_sum_parts(const double* __restrict__ parts, int count, int stride, int cols, double* out)
{
    const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (c >= cols) return;
    double s = 0;
    for (int j = lane; j < count; j += 32) s += parts[(long long)j * stride + c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) out[c] = s;
}

template <typename R>
__global__ void __launch_bounds__(kThreads) k_loss_sums(long long nn, const R* __restrict__ gm,
                                                         const R* __restrict__ tm, double* parts)
{
    __shared__ double red[32];
    double a = 0, b = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x) {
        a += (double)gm[i];
        b += (double)tm[4 * i + 3];
    }
    a = block_sum<R>(a, red);
    b = block_sum<R>(b, red);
    if (threadIdx.x == 0) {
        parts[2 * blockIdx.x] = a;
        parts[2 * blockIdx.x + 1] = b;
    }
}

// per-node loss and dL/dm (CompGraph.cpp:60-92)
template <typename R>
__global__ void __launch_bounds__(kThreads) k_loss_nodes(long long nn, const R* __restrict__ gm,
                                                          const R* __restrict__ tm, R* __restrict__ dLdm,
                                                          const double* acc, double* parts)
{
    __shared__ double red[32];
    const double eps = 1e-4, min_mass = 1e-3, eps_s = 1e-6;
    const double sc = (acc[1] + eps_s) / (acc[0] + eps_s);
    double loss = 0, gc = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x) {
        const double c = (double)gm[i];
        const double cms = sc * c;
        const double ld = log(cms + 1.0 + eps) - log((double)tm[4 * i + 3] + 1.0 + eps);
        loss += 0.5 * ld * ld;
        double gg = ld / (cms + 1.0 + eps);
        if (cms < min_mass) {
            const double diff = min_mass - cms;
            loss += diff * diff;
            gg += -2.0 * diff;
        }
        dLdm[i] = (R)(sc * gg);
        gc += gg * c;
    }
    loss = block_sum<R>(loss, red);
    gc = block_sum<R>(gc, red);
    if (threadIdx.x == 0) {
        parts[2 * blockIdx.x] = loss;
        parts[2 * blockIdx.x + 1] = gc;
    }
}

// dL/dx of the last layer (CompGraph.cpp:94-126); zeroes dL/dv, dL/dF, dL/dC
template <typename R, int K>
__global__ void __launch_bounds__(kThreads) k_loss_grad(KP<R> kp, int n, long long ld, const R* __restrict__ st,
                                                         const R* __restrict__ co, const R* __restrict__ tm,
                                                         const R* __restrict__ dLdm, const double* acc,
                                                         R* __restrict__ g)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    R x[3];
    load_planes(st + ST_X * ld, ld, p, 3, x);
    const R m = co[CO_M * ld + p];
    R corr = R(0);
    if (kp.exact) {
        const double eps_s = 1e-6;
        const double sc = (acc[1] + eps_s) / (acc[0] + eps_s);
        corr = (R)(acc[3] * (-sc / (acc[0] + eps_s)));
    }
    Stencil<R, K> sn;
    make_stencil<R, K>(x, kp.gmin, kp.dx, kp.inv_dx, sn, true);
    R a0 = 0, a1 = 0, a2 = 0;
    const R nidx = -kp.inv_dx;
#pragma unroll
    for (int a = 0; a < K; ++a)
#pragma unroll
        for (int b = 0; b < K; ++b)
#pragma unroll
            for (int c = 0; c < K; ++c) {
                const int i = sn.base[0] + a, j = sn.base[1] + b, k = sn.base[2] + c;
                if (!in_grid(kp, i, j, k)) continue;
                const long long nd = node_of(kp, i, j, k);
                const R pen = (kp.exact || tm[4 * nd + 3] > R(1e-12)) ? R(1) : R(5);
                const R f = pen * m * (dLdm[nd] + corr);
                a0 += f * nidx * sn.s[0][a] * sn.w[1][b] * sn.w[2][c];
                a1 += f * nidx * sn.w[0][a] * sn.s[1][b] * sn.w[2][c];
                a2 += f * nidx * sn.w[0][a] * sn.w[1][b] * sn.s[2][c];
            }
    g[(ST_X + 0) * ld + p] = a0;
    g[(ST_X + 1) * ld + p] = a1;
    g[(ST_X + 2) * ld + p] = a2;
#pragma unroll
    for (int q = 3; q < ST_N; ++q) g[(long long)q * ld + p] = R(0);
}

// ------------------------------------------------------------- volumes

template <typename R, int K>
__global__ void __launch_bounds__(kThreads) k_p2g_plain(KP<R> kp, int n, long long ld, const R* __restrict__ st,
                                                         const R* __restrict__ co, R* __restrict__ grid)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    R x[3], v[3], C[9];
    load_planes(st + ST_X * ld, ld, p, 3, x);
    load_planes(st + ST_V * ld, ld, p, 3, v);
    load_planes(st + ST_C * ld, ld, p, 9, C);
    const R m = co[CO_M * ld + p];
    Stencil<R, K> sn;
    make_stencil<R, K>(x, kp.gmin, kp.dx, kp.inv_dx, sn, false);
    walk_rotated<R, K>(sn, [&](int i, int j, int k, R w, R gx, R gy, R gz) {
        if (!in_grid(kp, i, j, k)) return;
        const long long nd = node_of(kp, i, j, k);
#pragma unroll
        for (int r = 0; r < 3; ++r)
            atomicAdd(&grid[nd * 4 + r], w * (m * v[r] + m * (C[r * 3] * gx + C[r * 3 + 1] * gy + C[r * 3 + 2] * gz)));
        atomicAdd(&grid[nd * 4 + 3], w * m);
    });
}

// CalculatePointCloudVolumes gather (ForwardSimulation.cpp:250-270)
template <typename R, int K>
__global__ void __launch_bounds__(kThreads) k_volumes(KP<R> kp, int n, long long ld, const R* __restrict__ st,
                                                       R* __restrict__ co, const R* __restrict__ grid)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    R x[3];
    load_planes(st + ST_X * ld, ld, p, 3, x);
    Stencil<R, K> sn;
    make_stencil<R, K>(x, kp.gmin, kp.dx, kp.inv_dx, sn, false);
    R mg = 0;
#pragma unroll
    for (int a = 0; a < K; ++a)
#pragma unroll
        for (int b = 0; b < K; ++b)
#pragma unroll
            for (int c = 0; c < K; ++c) {
                const int i = sn.base[0] + a, j = sn.base[1] + b, k = sn.base[2] + c;
                if (!in_grid(kp, i, j, k)) continue;
                mg += sn.w[0][a] * sn.w[1][b] * sn.w[2][c] * grid[node_of(kp, i, j, k) * 4 + 3];
            }
    const R cell = kp.dx * kp.dx * kp.dx;
    const R rho = mg / (cell > R(1e-12) ? cell : R(1e-12));
    co[CO_VOL * ld + p] = rho > R(1.1920928955078125e-07) ? co[CO_M * ld + p] / rho : R(0);
}

// ---------------------------------------------------------------- Adam

template <typename R>
__global__ void __launch_bounds__(kThreads) k_sumsq(int n, long long ld, const R* __restrict__ g, int planes,
                                                     double* parts)
{
    __shared__ double red[32];
    double s = 0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        for (int q = 0; q < planes; ++q) {
            const double v = (double)g[(long long)q * ld + p];
            s += v * v;
        }
    s = block_sum<R>(s, red);
    if (threadIdx.x == 0) parts[blockIdx.x] = s;
}

// Descend_Adam (PointCloud.cpp:83-147) with FP64 moments
template <typename R>
__global__ void __launch_bounds__(kThreads) k_adam(int n, long long ld, const R* __restrict__ gF, R* __restrict__ dfc,
                                                    double* __restrict__ mom, double* __restrict__ vec,
                                                    double* __restrict__ vmax, double alpha, double inv_gn,
                                                    double beta1, double beta2, double eps, double bc1, double bc2)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    double step[9], xo[9], sn = 0, xn = 0;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const long long k = (long long)i * ld + p;
        const double g = (double)gF[k] * inv_gn;
        const double m = beta1 * mom[k] + (1.0 - beta1) * g;
        const double v = beta2 * vec[k] + (1.0 - beta2) * g * g;
        mom[k] = m;
        vec[k] = v;
        const double vh = v / bc2;
        const double vm = vh > vmax[k] ? vh : vmax[k];
        vmax[k] = vm;
        double den = sqrt(vm);
        den = den < 1e-8 ? 1e-8 : den;
        step[i] = (m / bc1) / (den + eps);
        sn += step[i] * step[i];
        xo[i] = (double)dfc[k];
        xn += xo[i] * xo[i];
    }
    sn = sqrt(sn);
    xn = sqrt(xn);
    double cap = 5e-2 * (xn > 1.0 ? xn : 1.0);
    cap = cap < 5e-3 ? 5e-3 : cap;
    double scale = 1.0;
    if (sn > 0 && alpha * sn > cap) scale = cap / (alpha * sn);
    double small = 1e-3 * (xn > 1.0 ? xn : 1.0);
    small = small < 1e-4 ? 1e-4 : small;
    const bool near = alpha * sn <= small;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        double nx = xo[i] - alpha * step[i] * scale;
        if (near) nx = xo[i] + 0.2 * (nx - xo[i]);
        dfc[(long long)i * ld + p] = (R)nx;
    }
}

// ------------------------------------------------------------- utility

template <typename R, typename T>
__global__ void k_aos_to_planes(int n, int k, long long ld, const T* __restrict__ src, R* __restrict__ dst,
                                const int* __restrict__ perm)
{
    // slot p holds the caller's row perm[p] (identity without a permutation)
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * k) return;
    const int p = (int)(t % n), q = (int)(t / n);
    const long long row = perm ? perm[p] : p;
    dst[(long long)q * ld + p] = (R)src[row * k + q];
}

template <typename R, typename T>
__global__ void k_planes_to_aos(int n, int k, long long ld, const R* __restrict__ src, T* __restrict__ dst,
                                const int* __restrict__ perm)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * k) return;
    const int p = (int)(t % n), q = (int)(t / n);
    const long long row = perm ? perm[p] : p;
    dst[row * k + q] = (T)src[(long long)q * ld + p];
}

// dst slot i <- src slot order[i], plane by plane (the re-sort); one grid
// row per plane
template <typename R>
__global__ void k_gather_planes(int n, long long ld, const int* __restrict__ order, const R* __restrict__ src,
                                R* __restrict__ dst)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long q = blockIdx.y;
    dst[q * ld + i] = src[q * ld + order[i]];
}

template <typename R>
__global__ void k_axpy_planes(int n, int k, long long ld, R alpha, const R* __restrict__ x, R* __restrict__ y)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * k) return;
    const int q = (int)(t / n), p = (int)(t % n);
    y[(long long)q * ld + p] += alpha * x[(long long)q * ld + p];
}

template <typename R>
__global__ void k_fill_planes(int n, int k, long long ld, R value, R* __restrict__ y)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * k) return;
    const int q = (int)(t / n), p = (int)(t % n);
    y[(long long)q * ld + p] = value;
}

template <typename R>
__global__ void k_count_active(long long nn, const R* __restrict__ grid, unsigned long long* out)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool act = i < nn && grid[4 * i + 3] > R(0);
    unsigned b = __ballot_sync(0xffffffffu, act);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(out, (unsigned long long)__popc(b));
}

template <typename R>
__global__ void k_nonfinite(int n, int k, long long ld, const R* __restrict__ y, int* flag)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * k) return;
    const int q = (int)(t / n), p = (int)(t % n);
    if (!isfinite((double)y[(long long)q * ld + p])) *flag = 1;
}

template <typename R>
int tile_cap_for(const StepCfg& c)
{
    // shared float atomics are native; double tiles are not used (the plain
    // FP64 form scatters with global atomics)
    return sizeof(R) == 4 ? (c.tile_nodes >= 0 ? c.tile_nodes : g_tile_nodes) : 0;
}

// the G2P transpose's scatter tile: its own budget when the graph sets it,
// else P2G's; the P2G transpose's gather tile: its own budget, else 2048
template <typename R>
int adj_cap_for(const StepCfg& c)
{
    return sizeof(R) == 4 && c.adj_tile_nodes >= 0 ? c.adj_tile_nodes : tile_cap_for<R>(c);
}

template <typename R>
int gather_cap_for(const StepCfg& c)
{
    if (sizeof(R) != 4) return 0;
    return c.gather_tile_nodes >= 0 ? c.gather_tile_nodes : kGatherTileDefault;
}

inline int scatter_mode_of(const StepCfg& c) { return c.scatter_mode >= 0 ? c.scatter_mode : g_scatter_mode; }

}  // namespace

// ----------------------------------------------------------- launchers

template <typename R>
static void fill_table(const InstHost* h, int count, int kernel, std::vector<InstDev<R>>& out)
{
    out.resize(count);
    for (int i = 0; i < count; ++i) {
        InstDev<R>& d = out[i];
        d.dx = (R)h[i].dx;
        d.inv_dx = (R)(1.0 / h[i].dx);
        d.C0 = (R)((kernel == 0 ? 3.0 : 4.0) / (h[i].dx * h[i].dx));
        for (int a = 0; a < 3; ++a) {
            d.gmin[a] = (R)h[i].gmin[a];
            d.dims[a] = h[i].dims[a];
        }
        d.n = h[i].n;
        d.poff = h[i].poff;
        d.goff = h[i].goff;
    }
}

size_t inst_table_bytes(int count, int prec_bytes)
{
    return (size_t)count * (prec_bytes == 8 ? sizeof(InstDev<double>) : sizeof(InstDev<float>));
}

void make_inst_table(const InstHost* h, int count, int kernel, int prec_bytes, void* dst, cudaStream_t s)
{
    if (prec_bytes == 8) {
        std::vector<InstDev<double>> t;
        fill_table(h, count, kernel, t);
        cudaMemcpyAsync(dst, t.data(), t.size() * sizeof(t[0]), cudaMemcpyHostToDevice, s);
        cudaStreamSynchronize(s);
    } else {
        std::vector<InstDev<float>> t;
        fill_table(h, count, kernel, t);
        cudaMemcpyAsync(dst, t.data(), t.size() * sizeof(t[0]), cudaMemcpyHostToDevice, s);
        cudaStreamSynchronize(s);
    }
}

// Raise a kernel's dynamic shared-memory limit once (the attribute is
// persistent; setting it before every launch costs host time per launch).
template <typename KernelT>
void ensure_smem(KernelT* kernel, size_t bytes)
{
    // keyed by kernel address: instantiations can share one function type
    static std::unordered_map<const void*, size_t> done;
    size_t& cur = done[reinterpret_cast<const void*>(kernel)];
    if (bytes > cur) {
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        cur = bytes;
    }
}


template <typename R>
void launch_p2g(const StepCfg& c, int n, long long ld, const R* st, const R* dfc, const R* co, R* grid,
                cudaStream_t s)
{
    const int T = c.threads == 128 ? 128 : kThreads;
    if (n <= 0) return;
    const int cap = tile_cap_for<R>(c);
    auto kp = make_kp<R>(c);
    if constexpr (sizeof(R) == 4) {
        if (c.det()) {
            const FixArgs fx = make_fix(c);
            const size_t sm = seg_smem_bytes(T, cap, 4, true);
            if (c.kernel == 0) {
                ensure_smem(k_p2g_seg<4, true>, sm);
                counted();
                k_p2g_seg<4, true><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, co, grid, cap, fx);
            } else {
                ensure_smem(k_p2g_seg<3, true>, sm);
                counted();
                k_p2g_seg<3, true><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, co, grid, cap, fx);
            }
            return;
        }
        if (scatter_mode_of(c) == 1) {
            const size_t sm = seg_smem_bytes(T, cap, 4);
            const FixArgs fx{};
            if (c.kernel == 0) {
                ensure_smem(k_p2g_seg<4, false>, sm);
                counted();
                k_p2g_seg<4, false><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, co, grid, cap, fx);
            } else {
                ensure_smem(k_p2g_seg<3, false>, sm);
                counted();
                k_p2g_seg<3, false><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, co, grid, cap, fx);
            }
            return;
        }
    }
    const size_t sm = (size_t)cap * 4 * sizeof(R);
    counted();
    if (c.kernel == 0) k_p2g<R, 4><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, co, grid, cap);
    else k_p2g<R, 3><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, co, grid, cap);
}

bool g2p2g_applies(const StepCfg& c, int prec_bytes)
{
#if MPM_FUSE_G2P2G
    return prec_bytes == 4 && c.fuse && !c.det() && scatter_mode_of(c) == 1;
#else
    (void)c;
    (void)prec_bytes;
    return false;
#endif
}

void launch_g2p2g(const StepCfg& c, int n, long long ld, const float* st, const float* dfc, const float* co,
                  const float* grid, float* st1, float* trust, float* grid1, cudaStream_t s)
{
    const int T = c.threads == 128 ? 128 : kThreads;
    if (n <= 0) return;
    const int cap = tile_cap_for<float>(c);
    auto kp = make_kp<float>(c);
    const size_t sm = seg_smem_bytes(T, cap, 4);
    if (c.kernel == 0) {
        ensure_smem(k_g2p2g<4>, sm);
        counted();
        k_g2p2g<4><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, co, grid, st1, trust, grid1, cap);
    } else {
        ensure_smem(k_g2p2g<3>, sm);
        counted();
        k_g2p2g<3><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, co, grid, st1, trust, grid1, cap);
    }
}

template <typename R>
void launch_grid_update(const StepCfg& c, R* grid, cudaStream_t s, R* zero_next)
{
    const long long nn = c.nodes();
    if constexpr (sizeof(R) == 4) {
        if (c.det()) {
            if (zero_next) cudaMemsetAsync(zero_next, 0, sizeof(R) * 4 * nn, s);
            counted();
            k_grid_update_fix<<<nblocks(nn), kThreads, 0, s>>>(make_kp<R>(c), nn, make_fix(c), grid);
            return;
        }
    }
    counted();
    k_grid_update<R><<<nblocks(nn), kThreads, 0, s>>>(make_kp<R>(c), nn, grid, zero_next);
}

template <typename R>
void launch_g2p(const StepCfg& c, int n, long long ld, const R* st, const R* dfc, const R* grid, R* st1, R* trust,
                cudaStream_t s)
{
    const int T = c.threads == 128 ? 128 : kThreads;
    if (n <= 0) return;
    auto kp = make_kp<R>(c);
    counted();
    if (c.kernel == 0) k_g2p<R, 4><<<nblocks(n, T), T, 0, s>>>(kp, n, ld, st, dfc, grid, st1, trust);
    else k_g2p<R, 3><<<nblocks(n, T), T, 0, s>>>(kp, n, ld, st, dfc, grid, st1, trust);
}

template <typename R>
void launch_g2p_adj(const StepCfg& c, int n, long long ld, const R* st, const R* dfc, const R* st1, const R* g1,
                    const R* trust, R* adj, cudaStream_t s)
{
    const int T = c.threads == 128 ? 128 : kThreads;
    if (n <= 0) return;
    const int cap = adj_cap_for<R>(c);
    auto kp = make_kp<R>(c);
    if constexpr (sizeof(R) == 4) {
        if (c.det()) {
            // inputs of the scatter and their bound first, then the scatter
            const FixArgs fx = make_fix(c);
            cudaMemsetAsync(c.fix_ctl + 1, 0, 2 * sizeof(unsigned), s);
            const size_t sm = seg_smem_bytes(T, cap, 3, true);
            if (c.kernel == 0) {
                counted();
                k_g2p_adj_prep<4><<<nblocks(n, T), T, 0, s>>>(kp, n, ld, st, dfc, st1, g1, trust, fx, c.fix_scr);
                ensure_smem(k_g2p_adj_fix<4>, sm);
                counted();
                k_g2p_adj_fix<4><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, c.fix_scr, fx, cap);
            } else {
                counted();
                k_g2p_adj_prep<3><<<nblocks(n, T), T, 0, s>>>(kp, n, ld, st, dfc, st1, g1, trust, fx, c.fix_scr);
                ensure_smem(k_g2p_adj_fix<3>, sm);
                counted();
                k_g2p_adj_fix<3><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, c.fix_scr, fx, cap);
            }
            return;
        }
        if (scatter_mode_of(c) == 1) {
            const size_t sm = seg_smem_bytes(T, cap, 3);
            if (c.kernel == 0) {
                ensure_smem(k_g2p_adj_seg<4>, sm);
                counted();
                k_g2p_adj_seg<4><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, st1, g1, trust, adj, cap);
            } else {
                ensure_smem(k_g2p_adj_seg<3>, sm);
                counted();
                k_g2p_adj_seg<3><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, st1, g1, trust, adj, cap);
            }
            return;
        }
    }
    const size_t sm = (size_t)cap * 3 * sizeof(R);
    counted();
    if (c.kernel == 0) k_g2p_adj<R, 4><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, st1, g1, trust, adj, cap);
    else k_g2p_adj<R, 3><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, st1, g1, trust, adj, cap);
}

template <typename R>
void launch_grid_adj(const StepCfg& c, const R* grid, R* adj, cudaStream_t s, R* zero_next)
{
    const long long nn = c.nodes();
    if constexpr (sizeof(R) == 4) {
        if (c.det()) {
            if (zero_next) cudaMemsetAsync(zero_next, 0, sizeof(R) * 4 * nn, s);
            counted();
            k_grid_adj_fix<<<nblocks(nn), kThreads, 0, s>>>(make_kp<R>(c), nn, grid, make_fix(c), adj);
            return;
        }
    }
    counted();
    k_grid_adj<R><<<nblocks(nn), kThreads, 0, s>>>(make_kp<R>(c), nn, grid, adj, zero_next);
}

template <typename R>
void launch_p2g_adj(const StepCfg& c, int n, long long ld, const R* st, const R* dfc, const R* co, const R* st1,
                    const R* g1, const R* trust, const R* grid, const R* adj, R* g, R* gFt, R* glam, R* gmu,
                    cudaStream_t s)
{
    // 256 threads whatever the graph's block size: at its 255 registers two
    // 128-thread blocks per SM ran slower (0.579 against 0.532 ms per launch
    // on 2M particles)
    const int T = kThreads;
    if (n <= 0) return;
    auto kp = make_kp<R>(c);
    const int cap = gather_cap_for<R>(c);
    const size_t sm = (size_t)cap * 2 * sizeof(float4);
    if (c.kernel == 0) {
        ensure_smem(k_p2g_adj<R, 4>, sm);
        counted();
        k_p2g_adj<R, 4><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, co, st1, g1, trust, grid, adj, g, gFt,
                                                          glam, gmu, cap);
    } else {
        ensure_smem(k_p2g_adj<R, 3>, sm);
        counted();
        k_p2g_adj<R, 3><<<nblocks(n, T), T, sm, s>>>(kp, n, ld, st, dfc, co, st1, g1, trust, grid, adj, g, gFt,
                                                          glam, gmu, cap);
    }
}

template <typename R>
void launch_loss(const StepCfg& c, int n, long long ld, const R* st, const R* co, const R* target_m, R* gm, R* dLdm,
                 double* acc, R* g, cudaStream_t s)
{
    const long long nn = c.nodes();
    auto kp = make_kp<R>(c);
    bool fixed = false;
    if constexpr (sizeof(R) == 4) {
        if (c.det()) {
            const FixArgs fx = make_fix(c);
            launch_fix_prepare(c, n, ld, co, s);
            if (n > 0) {
                counted();
                if (c.kernel == 0) k_mass_p2g_fix<4><<<nblocks(n), kThreads, 0, s>>>(kp, n, ld, st, co, fx);
                else k_mass_p2g_fix<3><<<nblocks(n), kThreads, 0, s>>>(kp, n, ld, st, co, fx);
            }
            counted();
            k_fix_mass_out<<<nblocks(nn), kThreads, 0, s>>>(nn, fx, gm);
            fixed = true;
        }
    }
    if (!fixed) {
        cudaMemsetAsync(gm, 0, sizeof(R) * nn, s);
        if (n > 0) {
            counted();
            if (c.kernel == 0) k_mass_p2g<R, 4><<<nblocks(n), kThreads, 0, s>>>(kp, n, ld, st, co, gm);
            else k_mass_p2g<R, 3><<<nblocks(n), kThreads, 0, s>>>(kp, n, ld, st, co, gm);
        }
    }
    const int nb = (int)std::min<long long>(nblocks(nn), kRedParts);
    double* parts = acc + 8;
    counted();
    k_loss_sums<R><<<nb, kThreads, 0, s>>>(nn, gm, target_m, parts);
    counted();
    k_sum_parts<<<1, 64, 0, s>>>(parts, nb, 2, 2, acc);
    counted();
    k_loss_nodes<R><<<nb, kThreads, 0, s>>>(nn, gm, target_m, dLdm, acc, parts);
    counted();
    k_sum_parts<<<1, 64, 0, s>>>(parts, nb, 2, 2, acc + 2);
    if (n > 0) {
        counted();
        if (c.kernel == 0) k_loss_grad<R, 4><<<nblocks(n), kThreads, 0, s>>>(kp, n, ld, st, co, target_m, dLdm, acc, g);
        else k_loss_grad<R, 3><<<nblocks(n), kThreads, 0, s>>>(kp, n, ld, st, co, target_m, dLdm, acc, g);
    }
}

template <typename R>
void launch_p2g_plain(const StepCfg& c, int n, long long ld, const R* st, const R* co, R* grid, cudaStream_t s)
{
    if (n <= 0) return;
    auto kp = make_kp<R>(c);
    counted();
    if (c.kernel == 0) k_p2g_plain<R, 4><<<nblocks(n), kThreads, 0, s>>>(kp, n, ld, st, co, grid);
    else k_p2g_plain<R, 3><<<nblocks(n), kThreads, 0, s>>>(kp, n, ld, st, co, grid);
}

template <typename R>
void launch_volumes(const StepCfg& c, int n, long long ld, const R* st, R* co, const R* grid, cudaStream_t s)
{
    if (n <= 0) return;
    auto kp = make_kp<R>(c);
    counted();
    if (c.kernel == 0) k_volumes<R, 4><<<nblocks(n), kThreads, 0, s>>>(kp, n, ld, st, co, grid);
    else k_volumes<R, 3><<<nblocks(n), kThreads, 0, s>>>(kp, n, ld, st, co, grid);
}

template <typename R>
void launch_sumsq(int n, long long ld, const R* g, int plane0, int planes, double* acc, cudaStream_t s)
{
    if (n <= 0) {
        cudaMemsetAsync(acc, 0, sizeof(double), s);
        return;
    }
    const int nb = std::min(nblocks(n), kRedParts);
    counted();
    k_sumsq<R><<<nb, kThreads, 0, s>>>(n, ld, g + (long long)plane0 * ld, planes, acc + 8);
    counted();
    k_sum_parts<<<1, 32, 0, s>>>(acc + 8, nb, 1, 1, acc);
}

void launch_fix_prepare(const StepCfg& c, int n, long long ld, const float* co, cudaStream_t s)
{
    cudaMemsetAsync(c.fix_ctl, 0, 3 * sizeof(unsigned), s);
    counted();
    if (n > 0) k_fix_mass_max<<<nblocks(n), kThreads, 0, s>>>(n, ld, co, c.fix_ctl);
}

template <typename R>
void launch_adam(int n, long long ld, const R* gF, R* dfc, double* mom, double* vec, double* vmax, double alpha,
                 double inv_gn, double beta1, double beta2, double eps, int t, cudaStream_t s)
{
    if (n <= 0) return;
    const double bc1 = 1.0 - pow(beta1, t), bc2 = 1.0 - pow(beta2, t);
    counted();
    k_adam<R><<<nblocks(n), kThreads, 0, s>>>(n, ld, gF, dfc, mom, vec, vmax, alpha, inv_gn, beta1, beta2, eps, bc1,
                                               bc2);
}

template <typename R, typename T>
void launch_aos_to_planes(int n, int k, long long ld, const T* src, R* dst, cudaStream_t s, const int* perm)
{
    if (n <= 0) return;
    counted();
    k_aos_to_planes<R, T><<<nblocks((long long)n * k), kThreads, 0, s>>>(n, k, ld, src, dst, perm);
}

template <typename R, typename T>
void launch_planes_to_aos(int n, int k, long long ld, const R* src, T* dst, cudaStream_t s, const int* perm)
{
    if (n <= 0) return;
    counted();
    k_planes_to_aos<R, T><<<nblocks((long long)n * k), kThreads, 0, s>>>(n, k, ld, src, dst, perm);
}

template <typename R>
void launch_gather_planes(int n, int k, long long ld, const int* order, const R* src, R* dst, cudaStream_t s)
{
    if (n <= 0) return;
    counted();
    if (k <= 0) return;
    k_gather_planes<R><<<dim3(nblocks(n), k), kThreads, 0, s>>>(n, ld, order, src, dst);
}

template <typename R>
void launch_axpy_planes(int n, int k, long long ld, R alpha, const R* x, R* y, cudaStream_t s)
{
    if (n <= 0) return;
    counted();
    k_axpy_planes<R><<<nblocks((long long)n * k), kThreads, 0, s>>>(n, k, ld, alpha, x, y);
}

template <typename R>
void launch_fill_planes(int n, int k, long long ld, R value, R* y, cudaStream_t s)
{
    if (n <= 0) return;
    counted();
    k_fill_planes<R><<<nblocks((long long)n * k), kThreads, 0, s>>>(n, k, ld, value, y);
}

template <typename R>
void launch_count_active(const StepCfg& c, const R* grid, unsigned long long* out, cudaStream_t s)
{
    cudaMemsetAsync(out, 0, sizeof(unsigned long long), s);
    const long long nn = c.nodes();
    counted();
    k_count_active<R><<<nblocks(nn), kThreads, 0, s>>>(nn, grid, out);
}

template <typename R>
void launch_nonfinite(int n, int k, long long ld, const R* y, int* flag, cudaStream_t s)
{
    if (n <= 0) return;
    counted();
    k_nonfinite<R><<<nblocks((long long)n * k), kThreads, 0, s>>>(n, k, ld, y, flag);
}

#define MPM_INSTANTIATE(R)                                                                                         \
    template void launch_p2g<R>(const StepCfg&, int, long long, const R*, const R*, const R*, R*, cudaStream_t);   \
    template void launch_grid_update<R>(const StepCfg&, R*, cudaStream_t, R*);                                     \
    template void launch_g2p<R>(const StepCfg&, int, long long, const R*, const R*, const R*, R*, R*, cudaStream_t); \
    template void launch_g2p_adj<R>(const StepCfg&, int, long long, const R*, const R*, const R*, const R*,        \
                                    const R*, R*, cudaStream_t);                                                   \
    template void launch_grid_adj<R>(const StepCfg&, const R*, R*, cudaStream_t, R*);                              \
    template void launch_p2g_adj<R>(const StepCfg&, int, long long, const R*, const R*, const R*, const R*,        \
                                    const R*, const R*, const R*, const R*, R*, R*, R*, R*, cudaStream_t);         \
    template void launch_loss<R>(const StepCfg&, int, long long, const R*, const R*, const R*, R*, R*, double*, R*, \
                                 cudaStream_t);                                                                    \
    template void launch_p2g_plain<R>(const StepCfg&, int, long long, const R*, const R*, R*, cudaStream_t);       \
    template void launch_volumes<R>(const StepCfg&, int, long long, const R*, R*, const R*, cudaStream_t);         \
    template void launch_sumsq<R>(int, long long, const R*, int, int, double*, cudaStream_t);                     \
    template void launch_adam<R>(int, long long, const R*, R*, double*, double*, double*, double, double, double, \
                                 double, double, int, cudaStream_t);                                               \
    template void launch_aos_to_planes<R, float>(int, int, long long, const float*, R*, cudaStream_t, const int*); \
    template void launch_aos_to_planes<R, double>(int, int, long long, const double*, R*, cudaStream_t,           \
                                                  const int*);                                                      \
    template void launch_planes_to_aos<R, float>(int, int, long long, const R*, float*, cudaStream_t, const int*); \
    template void launch_planes_to_aos<R, double>(int, int, long long, const R*, double*, cudaStream_t,           \
                                                  const int*);                                                      \
    template void launch_gather_planes<R>(int, int, long long, const int*, const R*, R*, cudaStream_t);           \
    template void launch_axpy_planes<R>(int, int, long long, R, const R*, R*, cudaStream_t);                      \
    template void launch_fill_planes<R>(int, int, long long, R, R*, cudaStream_t);                                \
    template void launch_count_active<R>(const StepCfg&, const R*, unsigned long long*, cudaStream_t);             \
    template void launch_nonfinite<R>(int, int, long long, const R*, int*, cudaStream_t);

MPM_INSTANTIATE(float)
MPM_INSTANTIATE(double)

}  // namespace mpm
