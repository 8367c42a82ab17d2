/*
 * mpm.h -- C ABI of libmpm.so, the GB300 (sm_103a) differentiable MPM engine.
 *
 * The entry points replace the reference's pybind11 module `diffmpm_bindings`
 * (bind/bind.cpp:54-560) and the C++ classes it wraps (DiffMPMLib3D/
 * PointCloud.h, Grid.h, CompGraph.h).  Each declaration cites the reference
 * interface it stands in for.  Plain pointers and sizes only; no C++ or torch
 * types cross this boundary, and nothing throws across it.
 *
 * Conventions
 *   - Every function returns an int status: MPM_OK (0) or an MPM_ERR_* code;
 *     mpm_last_error() returns a message for the calling thread's last error.
 *   - Particle arrays are row-major: vectors (N,3), matrices (N,3,3).
 *   - Grid arrays are flattened with node (i,j,k) at i*ny*nz + j*nz + k
 *     (Grid.h:89-94).
 *   - `dtype` arguments select MPM_DTYPE_F32 or MPM_DTYPE_F64 for the caller's
 *     buffer; `on_device` says whether the buffer is CUDA device memory of the
 *     current device (else host memory).
 *   - Calls are synchronous with respect to the host unless stated otherwise;
 *     work runs on the object's CUDA stream (mpm_compgraph_set_stream).
 */
#ifndef MPM_H
#define MPM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status codes */
enum {
    MPM_OK = 0,
    MPM_ERR_ARG = 1,       /* invalid argument                      (RuntimeError) */
    MPM_ERR_SHAPE = 2,     /* array shape / size mismatch           (RuntimeError) */
    MPM_ERR_OOM = 3,       /* device allocation failed                              */
    MPM_ERR_NONFINITE = 4, /* NaN/Inf detected in state or loss                     */
    MPM_ERR_TIMEOUT = 5,   /* a bounded device wait gave up                         */
    MPM_ERR_CUDA = 6,      /* CUDA runtime error                                    */
    MPM_ERR_STATE = 7,     /* call not valid in the object's current state          */
    MPM_ERR_RANGE = 8      /* index out of range                    (IndexError)    */
};

enum { MPM_FP32 = 0, MPM_FP64 = 1 };             /* engine precision            */
enum { MPM_DTYPE_F32 = 0, MPM_DTYPE_F64 = 1 };   /* caller buffer element type  */
enum { MPM_ADJ_REFERENCE = 0, MPM_ADJ_EXACT = 1 };
enum { MPM_KERNEL_CUBIC = 0, MPM_KERNEL_QUADRATIC = 1 };
enum { MPM_MAT_FCR = 0, MPM_MAT_NEOHOOKEAN = 1 };

/* particle fields (MaterialPoint.h:17-46) */
enum {
    MPM_FIELD_X = 0,       /* (N,3)   position                                    */
    MPM_FIELD_V = 1,       /* (N,3)   velocity                                    */
    MPM_FIELD_F = 2,       /* (N,3,3) deformation gradient                        */
    MPM_FIELD_C = 3,       /* (N,3,3) APIC affine matrix                          */
    MPM_FIELD_DFC = 4,     /* (N,3,3) control dFc                                 */
    MPM_FIELD_F_TOTAL = 5, /* (N,3,3) F + dFc (read only)                         */
    MPM_FIELD_M = 6,       /* (N)     mass                                        */
    MPM_FIELD_VOL = 7,     /* (N)     rest volume                                 */
    MPM_FIELD_LAM = 8,     /* (N)     Lame lambda                                 */
    MPM_FIELD_MU = 9,      /* (N)     Lame mu                                     */
    MPM_FIELD_GRAD_X = 10, /* (N,3)   dL/dx                                       */
    MPM_FIELD_GRAD_V = 11, /* (N,3)   dL/dv                                       */
    MPM_FIELD_GRAD_F = 12, /* (N,3,3) dL/dF                                       */
    MPM_FIELD_GRAD_C = 13, /* (N,3,3) dL/dC                                       */
    MPM_FIELD_GRAD_DFC = 14,/* (N,3,3) dL/d(dFc), the control gradient (read only)*/
    MPM_FIELD_GRAD_LAM = 15,/* (N)    dL/dlambda accumulated over the backward    */
    MPM_FIELD_GRAD_MU = 16  /* (N)    dL/dmu accumulated over the backward        */
};

/* grid fields (GridNode.h:5-24) */
enum { MPM_GRID_MASS = 0, MPM_GRID_MOMENTUM = 1, MPM_GRID_VELOCITY = 2 };

/* simulation parameters; defaults = CompGraph's private members
 * (CompGraph.h:78-83) and ForwardSimulation.cpp:13 */
typedef struct mpm_params {
    double dt;             /* 1/120 */
    double drag;           /* 0.5   */
    double smoothing;      /* 0.1   */
    double f_ext[3];       /* 0     */
    double bulk_viscosity; /* 0.25  */
    double j_min;          /* 0.6 (trust region floor; <= 0 disables) */
} mpm_params;

typedef struct mpm_options {
    int precision;        /* MPM_FP32 (FP32 with FP64 guard) or MPM_FP64 (plain all-FP64)  */
    int adjoint;          /* MPM_ADJ_REFERENCE (term for term BackPropagation.cpp) or EXACT */
    int kernel;           /* MPM_KERNEL_CUBIC (reference) or MPM_KERNEL_QUADRATIC           */
    int material;         /* MPM_MAT_FCR (reference) or MPM_MAT_NEOHOOKEAN                  */
    int checkpoint_every; /* 1: keep every layer (reference tape); k > 1: keep every k-th
                             layer and recompute the others during the backward pass       */
    int deterministic;    /* FP32 only, no counterpart in the reference (which sums nodes
                             under `omp atomic`/`omp critical`, ForwardSimulation.cpp:26-80,
                             BackPropagation.cpp:36-55): 1 = P2G, the G2P transpose and the
                             loss's mass P2G sum node contributions in 64-bit fixed point,
                             so results are bitwise reproducible run to run and a
                             checkpointed backward recomputes the forward bit for bit      */
} mpm_options;

/* OptInput (bind.cpp:30-52) -- the fields run_optimization reads */
typedef struct mpm_opt_input {
    int num_timesteps, control_stride, max_gd_iters, max_ls_iters, current_episodes;
    double dt, drag, smoothing_factor, initial_alpha, gd_tol;
    double f_ext[3];
    /* additive: passes over the control steps (0: the reference's 3,
       CompGraph.cpp:245) */
    int passes;
} mpm_opt_input;

typedef struct mpm_pointcloud mpm_pointcloud;
typedef struct mpm_grid mpm_grid;
typedef struct mpm_compgraph mpm_compgraph;

/* ------------------------------------------------------------------- misc */
int mpm_version(void);
const char* mpm_last_error(void);
void mpm_default_params(mpm_params* p);
void mpm_default_options(mpm_options* o);
/* progress messages like the reference's std::cout lines (1 = on, default) */
void mpm_set_verbose(int verbose);
/* shared-memory node-tile budget of the scatter kernels (0, the default:
 * no tile, each cell group's sums go to global memory as float4 reductions) */
int mpm_set_tile_nodes(int nodes);
/* FP32 scatter strategy of P2G and the G2P transpose: 1 = segmented (one
 * warp per run of particles sharing a cell, one lane per stencil node; the
 * default), 0 = one thread per particle */
int mpm_set_scatter_mode(int mode);
/* No counterpart in the reference (whose ForwardTimeStep runs P2G, the grid
 * update and G2P one after another, ForwardSimulation.cpp:159-185): forward
 * passes in FP32 with float scatters run each step's G2P fused with the next
 * step's P2G, which then takes the new particle state from registers instead
 * of reading it back (1, the default); 0 runs the steps one by one.  The
 * computation is the same either way. */
int mpm_set_fused_steps(int on);
/* CalculateLameParameters (Elasticity.cpp:149-153; bind.cpp:540-544) */
int mpm_lame(double young, double poisson, double* lam, double* mu);

/* ------------------------------------------------------------- PointCloud */
/* PointCloud with n particles: x = v = C = dFc = 0, F = I, m = vol = lam = mu = 0
 * (MaterialPoint.h:17-31).  GeometryLoading.cpp:85-143 fills one from a mesh. */
int mpm_pointcloud_create(int n, int precision, mpm_pointcloud** out);
/* copy a field in (fields X..MU) */
int mpm_pointcloud_set(mpm_pointcloud* pc, int field, const void* src, int dtype, int on_device);
/* PointCloud::GetPoint* and bind.cpp:84-157 getters: copy a field out */
int mpm_pointcloud_get(const mpm_pointcloud* pc, int field, void* dst, int dtype, int on_device);
int mpm_pointcloud_size(const mpm_pointcloud* pc, int* n);
int mpm_pointcloud_precision(const mpm_pointcloud* pc, int* precision);
int mpm_pointcloud_release(mpm_pointcloud* pc);

/* ------------------------------------------------------------------- Grid */
/* Grid(int, int, int, float dx, Vec3 min) (Grid.cpp:7-26; bind.cpp:159-160) */
int mpm_grid_create(int nx, int ny, int nz, double dx, const double* min_point, int precision, mpm_grid** out);
int mpm_grid_info(const mpm_grid* g, int* dims, double* dx, double* min_point);
/* Grid::GetNodeMasses / GetNodeVelocities (Grid.cpp:236-270) */
int mpm_grid_get(const mpm_grid* g, int field, void* dst, int dtype, int on_device);
int mpm_grid_set(mpm_grid* g, int field, const void* src, int dtype, int on_device);
int mpm_grid_release(mpm_grid* g);

/* P2G(pc, grid, 0, 0) into the un-reset grid (bind.cpp:546-549) */
int mpm_p2g(mpm_pointcloud* pc, mpm_grid* g);
/* CalculatePointCloudVolumes (ForwardSimulation.cpp:234-271; bind.cpp:551-554) */
int mpm_calculate_point_cloud_volumes(mpm_pointcloud* pc, mpm_grid* g);
/* The inside test of GeometryLoading::GeneratePointCloudFromWatertightTriangleMesh
 * (GeometryLoading.cpp:57-77, libigl signed distance under the winding-number
 * sign; reached from load_point_cloud_from_obj, bind.cpp:531-538): the
 * generalized winding number of n_points points (n,3) w.r.t. n_tris
 * triangles given by their vertices (n_tris,3,3), into out (n doubles).
 * Points on the surface get exactly 0.5; |w| >= 0.5 is inside.  on_device:
 * the three arrays are device pointers (else host pointers). */
int mpm_winding_numbers(int n_points, const float* points, int n_tris, const float* tri_vertices, double* out,
                        int on_device, void* stream);

/* -------------------------------------------------------------- CompGraph */
/* CompGraph(pc, grid, target_grid) (CompGraph.cpp:21-28; bind.cpp:163-164):
 * deep-copies pc and grid, keeps a reference to target_grid. opt may be NULL. */
int mpm_compgraph_create(const mpm_pointcloud* pc, const mpm_grid* grid, mpm_grid* target_grid,
                         const mpm_options* opt, mpm_compgraph** out);
int mpm_compgraph_release(mpm_compgraph* cg);
/* No counterpart in the reference: a CompGraph
 * over `count` independent instances, each with its own particles and grid
 * (uneven sizes allowed), advanced together -- every kernel launch covers
 * all instances through per-instance particle and node offsets.  dt, drag,
 * smoothing, f_ext and the options are shared.  Layer views hold the
 * instances' particles concatenated; mpm_compgraph_batch_offsets gives where
 * instance i starts (particle_offsets[i], multiples of 256; its particles
 * are [particle_offsets[i], particle_offsets[i] + n_i)).  The mass loss is
 * not defined for batches. */
int mpm_compgraph_create_batch(const mpm_pointcloud* const* pcs, const mpm_grid* const* grids, int count,
                               const mpm_options* opt, mpm_compgraph** out);
/* count of instances (0: not a batch) and offsets (arrays of count+1; the
 * last particle entry is the end of the last instance's particles) */
int mpm_compgraph_batch_offsets(const mpm_compgraph* cg, int* count, long long* particle_offsets,
                                long long* node_offsets);
/* dt, drag, smoothing, f_ext (private in CompGraph.h:78-83; additive setter) */
int mpm_compgraph_set_params(mpm_compgraph* cg, const mpm_params* p);
int mpm_compgraph_get_params(const mpm_compgraph* cg, mpm_params* p);
int mpm_compgraph_get_options(const mpm_compgraph* cg, mpm_options* o);
/* run on a caller-owned cudaStream_t (NULL: the graph's own stream) */
int mpm_compgraph_set_stream(mpm_compgraph* cg, void* stream);
/* SetUpCompGraph (CompGraph.cpp:30-40; bind.cpp:345-347) */
int mpm_compgraph_set_up(mpm_compgraph* cg, int num_layers);
/* get_num_layers (bind.cpp:173-175) */
int mpm_compgraph_num_layers(const mpm_compgraph* cg, int* out);
/* ComputeForwardPass (CompGraph.cpp:131-141; bind.cpp:349-353) */
int mpm_compgraph_forward(mpm_compgraph* cg, int start_layer, int episode);
/* ComputeBackwardPass (CompGraph.cpp:143-211; bind.cpp:355-358) */
int mpm_compgraph_backward(mpm_compgraph* cg, int control_layer);
/* EndLayerMassLoss (CompGraph.cpp:42-129; bind.cpp:183-186) */
int mpm_compgraph_mass_loss(mpm_compgraph* cg, double* loss);
/* accumulate_render_grads (bind.cpp:189-279): float32 host arrays (n,3,3), (n,3) */
int mpm_compgraph_accumulate_render_grads(mpm_compgraph* cg, const float* dLdF, const float* dLdx, int n);
/* set/clear/has/info render gradients (bind.cpp:359-528) */
int mpm_compgraph_set_render_gradients(mpm_compgraph* cg, const float* dLdF, const float* dLdx, int n);
int mpm_compgraph_clear_render_gradients(mpm_compgraph* cg);
int mpm_compgraph_render_gradient_info(const mpm_compgraph* cg, int* has, int* num_points, double* grad_F_norm,
                                       double* grad_x_norm);
/* get_point_cloud / get_point_cloud_at_timestep (bind.cpp:176-180,320-343): a live
 * view of layer `layer`; release it with mpm_pointcloud_release */
int mpm_compgraph_layer(mpm_compgraph* cg, int layer, mpm_pointcloud** out);
/* promote_last_as_initial (bind.cpp:282-291) */
int mpm_compgraph_promote_last_as_initial(mpm_compgraph* cg, int carry_grid);
/* Compute_dLdF_Norm of a layer (PointCloud.cpp:24-35) over its control gradient */
int mpm_compgraph_grad_norm(mpm_compgraph* cg, int layer, double* out);
/* Descend_Adam on a layer's dFc (PointCloud.cpp:83-147), FP64 moments */
int mpm_compgraph_adam_step(mpm_compgraph* cg, int layer, double alpha, double grad_norm, double beta1,
                            double beta2, double eps, int timestep);
/* OptimizeSingleTimestep (CompGraph.cpp:369-465; bind.cpp:294-317) */
int mpm_compgraph_optimize_single_timestep(mpm_compgraph* cg, int timestep_idx, int max_gd_iters,
                                           int current_episode, double initial_alpha, int max_line_search_iters);
/* No counterpart in the reference, where OptimizeSingleTimestep's Adam step
 * counter is a function-local static shared by every CompGraph of the
 * process (CompGraph.cpp:396) that no caller can read or reset; this library
 * keeps the same process-wide counter.  *get (if get) receives it, then
 * *set (if set, >= 0) replaces it -- e.g. 0 to start a sequence of calls as
 * a fresh reference process would. */
int mpm_single_timestep_adam_step(int* get, const int* set);
/* OptimizeDefGradControlSequence (CompGraph.cpp:213-368; bind.cpp:165-172) */
int mpm_compgraph_run_optimization(mpm_compgraph* cg, const mpm_opt_input* opt);
/* No counterpart in the reference (which prints them): every loss the last
 * run_optimization evaluated, in order -- the initial loss, per gradient
 * step the loss before the step and each line-search trial, and the final
 * loss -- or, after optimize_single_timestep, the losses that call
 * evaluated (per gradient step the loss before the step and each
 * line-search trial).  *count receives the total; at most cap values are
 * copied. */
int mpm_compgraph_loss_history(const mpm_compgraph* cg, double* out, int cap, int* count);
/* forward and adjoint particle steps executed since load (recomputed
 * forward steps of checkpointed backward passes count as forward steps) */
void mpm_step_count(long long* forward_steps, long long* backward_steps);
/* number of grid nodes with mass > 0 in the forward grid of `layer` */
int mpm_compgraph_active_nodes(mpm_compgraph* cg, int layer, unsigned long long* out);
/* No counterpart in the reference (which only tests the loss with
 * std::isfinite, CompGraph.cpp:290-293): *flag = 1 if the state planes of
 * `layer` (x, v, C, F; with grads != 0 also its gradient planes) hold a NaN
 * or Inf, else 0.  One pass over the planes; the layer must be stored. */
int mpm_compgraph_nonfinite(mpm_compgraph* cg, int layer, int grads, int* flag);
/* number of grid nodes with mass > 0 in the forward grid of `layer` (the
 * last forward step's grid when the graph is checkpointed) -- see above */

/* PK_FixedCorotatedElasticity (Elasticity.cpp:45-55) and
 * d2_FCE_psi_dF2_mult_by_dF (Elasticity.cpp:57-117; the reference's only
 * callers are P_op_1 and Back_Timestep, ForwardSimulation.cpp:16-24,
 * BackPropagation.cpp:76-143), evaluated by the engine's own device code --
 * the functions P2G and its transpose inline -- on n matrices, so that the
 * branches a rollout rarely reaches can be checked: the FP64 guard near
 * inversion, the J clamp and the regularised rotation derivative.  precision
 * MPM_FP32 (FP32 with the FP64 guard; inputs rounded to float) or MPM_FP64;
 * material MPM_MAT_*; adjoint MPM_ADJ_REFERENCE (the reference's derivative)
 * or MPM_ADJ_EXACT.  Host arrays, double, row-major: F and G (n,3,3), lam
 * and mu (n); out: P (n,3,3) the stress, dP (n,3,3) the derivative of P at F
 * applied to G (the Hessian is symmetric, so this is also the VJP the
 * adjoint uses), branches (n ints, may be NULL): bit 0 FP64 SVD polar
 * decomposition, bit 1 FP64 det F / F^-T, bit 2 J clamped at 1e-6, bit 3
 * regularised rotation-derivative solve.  Synchronous; allocates its
 * device buffers. */
int mpm_constitutive(int n, int precision, int material, int adjoint, const double* F, const double* G,
                     const double* lam, const double* mu, double* P, double* dP, int* branches);

/* ---------------------------------------------------------- measurement */
/* kernel ids for the profiler */
enum { MPM_K_P2G = 0, MPM_K_GRID_UPDATE = 1, MPM_K_G2P = 2, MPM_K_G2P_ADJ = 3, MPM_K_GRID_ADJ = 4,
       MPM_K_P2G_ADJ = 5, MPM_K_LOSS = 6, MPM_K_ADAM = 7, MPM_K_NORM = 8,
       MPM_K_G2P2G = 10,    /* G2P of a step fused with the next step's P2G */
       MPM_K_RESORT = 11,   /* in-rollout re-sort at a segment start (sort, gathers) */
       MPM_K_BOUNDARY = 12, /* backward pass: gradients carried across a re-sorted boundary */
       MPM_K_COUNT = 13 };
/* record CUDA events around every kernel launch on its stream (1 = on) */
int mpm_profile_enable(int on);
/* which kernel ids the profiler times while on: bit k = id k (default all).
   Each timed launch adds two event records to its stream (graph nodes in a
   recorded pass); a changed selection or on/off state re-records a pass. */
int mpm_profile_select(unsigned long long mask);
int mpm_profile_reset(void);
/* launches and summed device time of one kernel id since the last reset */
int mpm_profile_query(int kernel, long long* launches, double* total_ms);
const char* mpm_kernel_name(int kernel);
/* number of engine kernels launched since the library was loaded */
long long mpm_launch_count(void);

/* per-graph scatter strategy and node-tile budget (-1: library defaults,
 * see mpm_set_scatter_mode / mpm_set_tile_nodes) */
int mpm_compgraph_set_tuning(mpm_compgraph* cg, int tile_nodes, int scatter_mode);
int mpm_compgraph_get_tuning(const mpm_compgraph* cg, int* tile_nodes, int* scatter_mode);
/* node-tile budgets of the adjoint kernels (FP32): the G2P transpose's
 * scatter and the P2G transpose's gather, whose best sizes differ from P2G's
 * (-1, the default: the scatter follows the set_tuning budget, the gather
 * stages 2048 nodes; 0..2816 nodes); get returns the budgets in effect */
int mpm_compgraph_set_adjoint_tiles(mpm_compgraph* cg, int scatter_nodes, int gather_nodes);
/* No counterpart in the reference: threads per block of the step kernels
 * (P2G, the fused G2P->P2G, G2P and the G2P transpose; the P2G transpose
 * keeps 256), 128 or 256 (-1: 256, the default).  Each thread takes one
 * particle, so this is also the particles per block; the segmented
 * scatter's node tile covers one block's particles. */
int mpm_compgraph_set_block_threads(mpm_compgraph* cg, int threads);
int mpm_compgraph_get_block_threads(const mpm_compgraph* cg, int* threads);
int mpm_compgraph_get_adjoint_tiles(const mpm_compgraph* cg, int* scatter_nodes, int* gather_nodes);
/* No counterpart in the reference: time `steps`-step forward+backward passes
 * of a scratch copy of this graph (layer 0's state) for each candidate
 * scatter strategy and P2G tile budget, then for each budget of the G2P
 * transpose's scatter tile and of the P2G transpose's gather tile, then for
 * 128 against 256 threads (and particles) per block (one knob at a time,
 * the others held), keep the fastest for this graph and return P2G's
 * choice (best_ms: one timed forward+backward of the winner; the adjoint
 * budgets: mpm_compgraph_get_adjoint_tiles; the block size:
 * mpm_compgraph_get_block_threads) */
int mpm_compgraph_autotune(mpm_compgraph* cg, int steps, int* best_tile, int* best_mode, double* best_ms);
/* the same, timing the candidates from the state of `layer` (a stored layer
 * after a forward pass).  A layer deep in a rollout has drifted from the
 * cell order of the set-up sort, which favours larger scatter tiles than
 * layer 0 does. */
int mpm_compgraph_autotune_from(mpm_compgraph* cg, int layer, int steps, int* best_tile, int* best_mode,
                                double* best_ms);
/* record forward/backward passes as CUDA graphs and replay them (1 = on,
 * the default): a pass is recorded the second time it runs with the same
 * buffers and parameters and replayed from then on */
int mpm_compgraph_use_graphs(mpm_compgraph* cg, int on);
/* No counterpart in the reference: switch mpm_options.deterministic of an
 * existing graph (MPM_ERR_ARG for FP64 graphs).  A pass whose node sums leave
 * the fixed-point range (a non-finite or exploding state) fails with
 * MPM_ERR_NONFINITE. */
int mpm_compgraph_set_deterministic(mpm_compgraph* cg, int on);
/* No counterpart in the reference (whose particles keep their order): order
 * the graph's particles by (instance, grid cell) of layer 0's positions, the
 * order the scatter and gather kernels run fastest in.  Every layer's planes
 * move; the graph keeps the permutation and every get/set goes through it,
 * so callers see their own particle order unchanged.  set_up_comp_graph (and
 * so run_optimization) re-sorts by default; mpm_compgraph_set_resort(cg, 0)
 * turns that off. */
int mpm_compgraph_resort(mpm_compgraph* cg);
int mpm_compgraph_set_resort(mpm_compgraph* cg, int on);
/* No counterpart in the reference: re-sort inside a rollout.  A forward pass
 * re-sorts the particles by cell at every `layers`-th layer after its start
 * (rounded up to a multiple of the checkpoint interval: segment starts), so
 * the particles stay in cell order as they move; each segment keeps its own
 * order and the backward pass carries the gradients across the boundaries.
 * Gets and sets still see the caller's order.  -1 (the default): the
 * checkpoint interval, or 20 with the full tape, for graphs of at least 2^16
 * particles, else never; 0: never.  Results equal those without re-sorting
 * up to the order of float additions (bit for bit with deterministic
 * scatters).  Gradients of layers other than the last and the control layer
 * are the backward pass's output: a forward pass leaves them undefined. */
int mpm_compgraph_set_resort_every(mpm_compgraph* cg, int layers);
/* the interval in effect (0: never) */
int mpm_compgraph_get_resort_every(const mpm_compgraph* cg, int* layers);
/* The particle order of a layer: slot p holds the caller's particle out[p]
 * (n ints).  Diagnostics; no counterpart in the reference. */
int mpm_compgraph_particle_order(mpm_compgraph* cg, int layer, int* out);
/* accumulate dL/dlambda and dL/dmu per particle over the next backward
 * passes; read them from the control layer's MPM_FIELD_GRAD_LAM/GRAD_MU */
int mpm_compgraph_enable_lame_grads(mpm_compgraph* cg, int on);
/* wait for all work queued on the graph's stream */
int mpm_compgraph_synchronize(mpm_compgraph* cg);

/* ------------------------------------------------- allocation-free variant */
/* No counterpart in the reference.  The end-layer mass loss of
 * mpm_compgraph_mass_loss (EndLayerMassLoss, FP32, cubic kernel) for callers
 * that cannot allocate device memory: code that must stay inside a fixed
 * device-memory budget it may not grow, or a host runtime that owns every
 * device allocation of the process.  The caller passes device buffers: x
 * (n,3) and m (n) particle positions and masses, target_mass (nx*ny*nz) node
 * masses; dLdx (n,3) receives dL/dx and *loss (host) the loss.  exact = 1
 * selects the exact derivative of the loss, 0 the reference's own.  The
 * function calls no cudaMalloc, cudaFree or other allocating routine: its
 * scratch (grid mass, dL/dm, FP64 sums) is a file-scope __device__ array of
 * 256 + 8 * MPM_NOALLOC_MAX_NODES bytes (about 8 MB).  CUDA loads the array
 * into a device's context with the first call on that device (lazy module
 * loading, the default), and that first call is where its memory is
 * allocated; it stays until the context is destroyed.  So make one call per
 * device ahead of time, outside the restricted context (any valid inputs; n
 * may be 0), or run the process with CUDA_MODULE_LOADING=EAGER; every later
 * call allocates nothing.  Grids with more than MPM_NOALLOC_MAX_NODES nodes
 * are rejected with MPM_ERR_SHAPE.  All calls share the one array, which
 * keeps the previous call's contents (the function clears what it
 * accumulates): calls that overlap on the GPU race.  Work is ordered on
 * `stream` (a cudaStream_t, NULL = legacy default stream) and the call is
 * synchronous -- it returns after the loss has been copied back -- so it
 * must not be made from a stream callback (cudaLaunchHostFunc), and a stream
 * that is being captured is refused with MPM_ERR_STATE. */
#define MPM_NOALLOC_MAX_NODES (1 << 20)
int mpm_mass_loss_noalloc(int n, const float* x, const float* m, const float* target_mass, const int* dims,
                          double dx, const double* min_point, int exact, float* dLdx, double* loss, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MPM_H */
