// ref_driver.cpp -- C entry points over the reference DiffMPMLib3D sources.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_oracle.py compiles this file
// together with the reference's own DiffMPMLib3D/*.cpp (read from the
// reference tree, never copied into this repository) into
// oracle/_ref/libref32.so (float, as shipped) and oracle/_ref/libref64.so
// (the same sources with float mechanically widened to double).  Tests use
// these libraries to pin the FP64 restatement in oracle/mpm_oracle.c and to
// generate the golden fixtures under tests/golden/.
//
// All arrays are double, row-major: vectors (N,3), matrices (N,3,3); grid
// node (i,j,k) at i*dy*dz + j*dz + k.
#include "pch.h"
#include "PointCloud.h"
#include "Grid.h"
#include "ForwardSimulation.h"
#include "BackPropagation.h"
#include "CompGraph.h"
#include "Elasticity.h"
#include "GeometryLoading.h"

#include <cstdio>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>

using namespace DiffMPMLib3D;
typedef Vec3::Scalar Real;

namespace {

Vec3 vec(const double* a) { return Vec3((Real)a[0], (Real)a[1], (Real)a[2]); }

Mat3 mat(const double* a)
{
    Mat3 M;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) M(r, c) = (Real)a[r * 3 + c];
    return M;
}

void put(const Vec3& v, double* a)
{
    for (int r = 0; r < 3; ++r) a[r] = (double)v[r];
}

void put(const Mat3& M, double* a)
{
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) a[r * 3 + c] = (double)M(r, c);
}

std::shared_ptr<PointCloud> make_pc(int n, const double* x, const double* v, const double* C, const double* F,
                                    const double* dFc, const double* m, const double* vol, const double* lam,
                                    const double* mu)
{
    auto pc = std::make_shared<PointCloud>();
    pc->points.resize(n);
    for (int p = 0; p < n; ++p) {
        MaterialPoint& mp = pc->points[p];
        mp.x = vec(x + 3 * p);
        mp.v = v ? vec(v + 3 * p) : Vec3::Zero();
        mp.C = C ? mat(C + 9 * p) : Mat3::Zero();
        mp.F = F ? mat(F + 9 * p) : Mat3::Identity();
        mp.dFc = dFc ? mat(dFc + 9 * p) : Mat3::Zero();
        mp.m = (Real)m[p];
        mp.vol = vol ? (Real)vol[p] : (Real)0;
        mp.lam = lam ? (Real)lam[p] : (Real)0;
        mp.mu = mu ? (Real)mu[p] : (Real)0;
    }
    return pc;
}

std::shared_ptr<Grid> make_grid(const int* dims, double dx, const double* mn)
{
    // The reference Grid constructor prints its size; keep stdout clean.
    std::streambuf* old = std::cout.rdbuf(nullptr);
    auto g = std::make_shared<Grid>(dims[0], dims[1], dims[2], (Real)dx, vec(mn));
    std::cout.rdbuf(old);
    return g;
}

}  // namespace

extern "C" {

int ref_real_size(void) { return (int)sizeof(Real); }

void ref_pk(const double* F, double lam, double mu, double* P)
{
    put(PK_FixedCorotatedElasticity(mat(F), (Real)lam, (Real)mu), P);
}

void ref_hvp(const double* F, double lam, double mu, const double* dF, double* out)
{
    put(d2_FCE_psi_dF2_mult_by_dF(mat(F), (Real)lam, (Real)mu, mat(dF)), out);
}

void ref_lame(double E, double nu, double* lam, double* mu)
{
    Real l, m;
    CalculateLameParameters((Real)E, (Real)nu, l, m);
    *lam = l;
    *mu = m;
}

// ForwardTimeStep (ForwardSimulation.cpp:159-185) on one layer pair.
int ref_forward_step(const int* dims, double dx, const double* mn, double dt, double drag, double smoothing,
                     const double* fext, int n, const double* x, const double* v, const double* C, const double* F,
                     const double* dFc, const double* m, const double* vol, const double* lam, const double* mu,
                     double* x1, double* v1, double* C1, double* F1, double* gm, double* gv)
{
    auto curr = make_pc(n, x, v, C, F, dFc, m, vol, lam, mu);
    auto next = std::make_shared<PointCloud>(*curr);
    auto grid = make_grid(dims, dx, mn);
    SingleThreadMPM::ForwardTimeStep(*next, *curr, *grid, (Real)smoothing, (Real)dt, (Real)drag, vec(fext), 0);
    for (int p = 0; p < n; ++p) {
        put(next->points[p].x, x1 + 3 * p);
        put(next->points[p].v, v1 + 3 * p);
        put(next->points[p].C, C1 + 9 * p);
        put(next->points[p].F, F1 + 9 * p);
    }
    size_t nn = grid->nodes.size();
    for (size_t i = 0; i < nn; ++i) {
        gm[i] = grid->nodes[i].m;
        put(grid->nodes[i].v, gv + 3 * i);
    }
    return 0;
}

// Back_Timestep (BackPropagation.cpp:9-144) with the reset that
// CompGraph::ComputeBackwardPass performs first (CompGraph.cpp:199-205).
int ref_backward_step(const int* dims, double dx, const double* mn, double dt, double drag, double smoothing, int n,
                      const double* x, const double* v, const double* C, const double* F, const double* dFc,
                      const double* m, const double* vol, const double* lam, const double* mu, const double* C1,
                      const double* gm, const double* gv_node, const double* gx1, const double* gv1,
                      const double* gF1, const double* gC1, double* gx, double* gv, double* gF, double* gC)
{
    CompGraphLayer ln, ln1;
    ln.point_cloud = make_pc(n, x, v, C, F, dFc, m, vol, lam, mu);
    SingleThreadMPM::P_op_1(*ln.point_cloud, 0);  // P as the forward stored it
    ln.grid = make_grid(dims, dx, mn);
    for (size_t i = 0; i < ln.grid->nodes.size(); ++i) {
        ln.grid->nodes[i].m = (Real)gm[i];
        ln.grid->nodes[i].v = vec(gv_node + 3 * i);
    }
    ln1.point_cloud = std::make_shared<PointCloud>(*ln.point_cloud);
    for (int p = 0; p < n; ++p) {
        MaterialPoint& q = ln1.point_cloud->points[p];
        q.C = mat(C1 + 9 * p);
        q.dLdx = vec(gx1 + 3 * p);
        q.dLdv = vec(gv1 + 3 * p);
        q.dLdF = mat(gF1 + 9 * p);
        q.dLdC = mat(gC1 + 9 * p);
    }
    ln1.grid = ln.grid;
    ln.grid->ResetGradients();
    ln.point_cloud->ResetGradients();
    Back_Timestep(ln1, ln, (Real)drag, (Real)dt, (Real)smoothing);
    for (int p = 0; p < n; ++p) {
        const MaterialPoint& q = ln.point_cloud->points[p];
        put(q.dLdx, gx + 3 * p);
        put(q.dLdv, gv + 3 * p);
        put(q.dLdF, gF + 9 * p);
        put(q.dLdC, gC + 9 * p);
    }
    return 0;
}

// EndLayerMassLoss (CompGraph.cpp:42-129) on a one-layer graph.
double ref_mass_loss(const int* dims, double dx, const double* mn, int n, const double* x, const double* m,
                     const double* target_m, double* gm, double* dLdm, double* gx)
{
    auto pc = make_pc(n, x, nullptr, nullptr, nullptr, nullptr, m, nullptr, nullptr, nullptr);
    auto grid = make_grid(dims, dx, mn);
    auto tgt = make_grid(dims, dx, mn);
    for (size_t i = 0; i < tgt->nodes.size(); ++i) tgt->nodes[i].m = (Real)target_m[i];
    std::streambuf* old = std::cout.rdbuf(nullptr);
    CompGraph cg(pc, grid, tgt);
    std::cout.rdbuf(old);
    double loss = cg.EndLayerMassLoss();
    const Grid& g = *cg.layers.back().grid;
    for (size_t i = 0; i < g.nodes.size(); ++i) {
        gm[i] = g.nodes[i].m;
        dLdm[i] = g.nodes[i].dLdm;
    }
    const PointCloud& q = *cg.layers.back().point_cloud;
    for (int p = 0; p < n; ++p) put(q.points[p].dLdx, gx + 3 * p);
    return loss;
}

// Descend_Adam (PointCloud.cpp:83-147) and Compute_dLdF_Norm (PointCloud.cpp:24-35).
double ref_adam(int n, const double* dLdF, double* dFc, double* mom, double* vec_, double* vmax, double alpha,
                double beta1, double beta2, double eps, int timestep)
{
    PointCloud pc;
    pc.points.resize(n);
    for (int p = 0; p < n; ++p) {
        MaterialPoint& q = pc.points[p];
        q.dLdF = mat(dLdF + 9 * p);
        q.dFc = mat(dFc + 9 * p);
        q.momentum = mat(mom + 9 * p);
        q.vector = mat(vec_ + 9 * p);
        q.vector_max = mat(vmax + 9 * p);
    }
    Real gn = pc.Compute_dLdF_Norm();
    Real gnorm = gn > (Real)1e-12 ? gn : (Real)1e-12;
    pc.Descend_Adam((Real)alpha, gnorm, (Real)beta1, (Real)beta2, (Real)eps, timestep);
    for (int p = 0; p < n; ++p) {
        const MaterialPoint& q = pc.points[p];
        put(q.dFc, dFc + 9 * p);
        put(q.momentum, mom + 9 * p);
        put(q.vector, vec_ + 9 * p);
        put(q.vector_max, vmax + 9 * p);
    }
    return (double)gn;
}

// CalculatePointCloudVolumes (ForwardSimulation.cpp:234-271) into a grid that
// already holds gm/gp.
void ref_volumes(const int* dims, double dx, const double* mn, int n, const double* x, const double* v,
                 const double* C, const double* m, double* gm, double* gp, double* vol)
{
    auto pc = make_pc(n, x, v, C, nullptr, nullptr, m, nullptr, nullptr, nullptr);
    auto grid = make_grid(dims, dx, mn);
    for (size_t i = 0; i < grid->nodes.size(); ++i) {
        grid->nodes[i].m = (Real)gm[i];
        grid->nodes[i].p = vec(gp + 3 * i);
    }
    SingleThreadMPM::CalculatePointCloudVolumes(*pc, *grid);
    for (int p = 0; p < n; ++p) vol[p] = pc->points[p].vol;
    for (size_t i = 0; i < grid->nodes.size(); ++i) {
        gm[i] = grid->nodes[i].m;
        put(grid->nodes[i].p, gp + 3 * i);
    }
}

// Full tape: forward T steps (CompGraph::ComputeForwardPass) and backward to
// layer 0 (CompGraph::ComputeBackwardPass) with a last-layer dL/dx seed.
// Returns the layer-0 gradients and the final positions.  Used to time the
// reference CPU path and to generate multi-step golden vectors.
int ref_rollout(const int* dims, double dx, const double* mn, double dt, double drag, double smoothing,
                const double* fext, int n, int T, const double* x0, const double* v0, const double* F0,
                const double* dFc0, const double* m, const double* vol, const double* lam, const double* mu,
                const double* seed_gx, double* xT, double* gx0, double* gv0, double* gF0, double* gC0,
                double* t_fwd, double* t_bwd)
{
    auto pc = make_pc(n, x0, v0, nullptr, F0, dFc0, m, vol, lam, mu);
    auto grid = make_grid(dims, dx, mn);
    std::streambuf* old = std::cout.rdbuf(nullptr);
    CompGraph cg(pc, grid, grid);
    cg.dt = (Real)dt;
    cg.drag = (Real)drag;
    cg.smoothing_factor = (Real)smoothing;
    cg.f_ext = vec(fext);
    cg.SetUpCompGraph(T + 1);
    double t0 = omp_get_wtime();
    cg.ComputeForwardPass(0, 0);
    double t1 = omp_get_wtime();
    PointCloud& last = *cg.layers.back().point_cloud;
    for (int p = 0; p < n; ++p) {
        last.points[p].ResetGradients();
        last.points[p].dLdx = vec(seed_gx + 3 * p);
    }
    double t2 = omp_get_wtime();
    cg.ComputeBackwardPass(0);
    double t3 = omp_get_wtime();
    std::cout.rdbuf(old);
    if (t_fwd) *t_fwd = t1 - t0;
    if (t_bwd) *t_bwd = t3 - t2;
    for (int p = 0; p < n; ++p) {
        put(last.points[p].x, xT + 3 * p);
        const MaterialPoint& q = cg.layers[0].point_cloud->points[p];
        put(q.dLdx, gx0 + 3 * p);
        put(q.dLdv, gv0 + 3 * p);
        put(q.dLdF, gF0 + 9 * p);
        put(q.dLdC, gC0 + 9 * p);
    }
    return 0;
}

// OptimizeDefGradControlSequence (CompGraph.cpp:213-368) as shipped (3
// passes, reference adjoint) on a graph built from arrays.  Returns the
// final loss and writes the control dFc of every layer (L = num_steps
// layers, (L,N,3,3)) and the last layer's positions.  The optimiser's own
// progress lines (initial/final loss) go to `log` (cap bytes) when given.
double ref_optimize(const int* dims, double dx, const double* mn, double dt, double drag, double smoothing,
                    const double* fext, int n, const double* x0, const double* v0, const double* F0,
                    const double* m, const double* vol, const double* lam, const double* mu, const double* target_m,
                    int num_steps, int control_stride, int max_gd, int max_ls, double alpha, double gd_tol,
                    double* dFc_out, double* xT, char* log, int cap)
{
    auto pc = make_pc(n, x0, v0, nullptr, F0, nullptr, m, vol, lam, mu);
    auto grid = make_grid(dims, dx, mn);
    auto tgt = make_grid(dims, dx, mn);
    for (size_t i = 0; i < tgt->nodes.size(); ++i) tgt->nodes[i].m = (Real)target_m[i];
    std::ostringstream text;
    std::streambuf* old = std::cout.rdbuf(text.rdbuf());
    CompGraph cg(pc, grid, tgt);
    cg.OptimizeDefGradControlSequence(num_steps, (Real)dt, (Real)drag, vec(fext), control_stride, max_gd, max_ls,
                                      (Real)alpha, (Real)gd_tol, (Real)smoothing, 0);
    double loss = cg.EndLayerMassLoss();
    std::cout.rdbuf(old);
    if (log && cap > 0) {
        const std::string t = text.str();
        const size_t k = std::min(t.size(), (size_t)cap - 1);
        memcpy(log, t.data(), k);
        log[k] = 0;
    }
    for (size_t l = 0; l < cg.layers.size(); ++l)
        for (int p = 0; p < n; ++p) put(cg.layers[l].point_cloud->points[p].dFc, dFc_out + (l * n + p) * 9);
    for (int p = 0; p < n; ++p) put(cg.layers.back().point_cloud->points[p].x, xT + 3 * p);
    return loss;
}

// The E2E path of run.py (run.py:1146-1149,665,686) on a graph built from
// arrays: SetUpCompGraph(num_layers), ComputeForwardPass(0, 0), optional
// render gradients (the members set_render_gradients fills, bind.cpp:359-451),
// then `calls` OptimizeSingleTimestep calls (CompGraph.cpp:369-465), call c
// with (t[c], max_gd[c], episode 0, alpha[c], max_ls[c]).  After each call it
// records every layer's dFc (dFc_out: (calls, L, N, 3, 3)), the last layer's
// positions (xT: (calls, N, 3)) and EndLayerMassLoss (loss: (calls)).  The
// optimiser's own lines go to `log` (cap bytes).  OptimizeSingleTimestep's
// Adam step counter is a function-local static (CompGraph.cpp:396): it
// starts at 0 in a fresh process and carries over between calls.
int ref_optimize_single(const int* dims, double dx, const double* mn, double dt, double drag, double smoothing,
                        int n, const double* x0, const double* v0, const double* F0, const double* m,
                        const double* vol, const double* lam, const double* mu, const double* target_m,
                        int num_layers, const float* render_dLdF, const float* render_dLdx, int calls,
                        const int* t, const int* max_gd, const double* alpha, const int* max_ls, double* dFc_out,
                        double* xT, double* loss, char* log, int cap)
{
    auto pc = make_pc(n, x0, v0, nullptr, F0, nullptr, m, vol, lam, mu);
    auto grid = make_grid(dims, dx, mn);
    auto tgt = make_grid(dims, dx, mn);
    for (size_t i = 0; i < tgt->nodes.size(); ++i) tgt->nodes[i].m = (Real)target_m[i];
    std::ostringstream text;
    std::streambuf* old = std::cout.rdbuf(text.rdbuf());
    CompGraph cg(pc, grid, tgt);
    cg.dt = (Real)dt;
    cg.drag = (Real)drag;
    cg.smoothing_factor = (Real)smoothing;
    cg.SetUpCompGraph(num_layers);
    cg.ComputeForwardPass(0, 0);
    if (render_dLdF && render_dLdx) {
        cg.stored_render_grad_F_.assign(render_dLdF, render_dLdF + 9 * (size_t)n);
        cg.stored_render_grad_x_.assign(render_dLdx, render_dLdx + 3 * (size_t)n);
        cg.render_grad_num_points_ = (size_t)n;
        cg.has_render_grads_ = true;
    }
    const size_t L = cg.layers.size();
    for (int c = 0; c < calls; ++c) {
        cg.OptimizeSingleTimestep(t[c], max_gd[c], 0, (Real)alpha[c], max_ls[c]);
        for (size_t l = 0; l < L; ++l)
            for (int p = 0; p < n; ++p)
                put(cg.layers[l].point_cloud->points[p].dFc, dFc_out + (((size_t)c * L + l) * n + p) * 9);
        for (int p = 0; p < n; ++p) put(cg.layers.back().point_cloud->points[p].x, xT + ((size_t)c * n + p) * 3);
        loss[c] = cg.EndLayerMassLoss();
    }
    std::cout.rdbuf(old);
    if (log && cap > 0) {
        const std::string s = text.str();
        const size_t k = std::min(s.size(), (size_t)cap - 1);
        memcpy(log, s.data(), k);
        log[k] = 0;
    }
    return 0;
}

// GeneratePointCloudFromWatertightTriangleMesh (GeometryLoading.cpp:10-83)
// over the mesh's bounding box, as LoadMPMPointCloudFromObj calls it
// (GeometryLoading.cpp:103-118): writes up to cap points (cap,3) and returns
// how many the reference keeps.
int ref_sample_mesh(const double* V, int nv, const int* F, int nt, double dx, double* out, int cap)
{
    Eigen::Matrix<Real, Eigen::Dynamic, Eigen::Dynamic> Vm(nv, 3);
    Eigen::MatrixXi Fm(nt, 3);
    for (int i = 0; i < nv; ++i)
        for (int j = 0; j < 3; ++j) Vm(i, j) = (Real)V[3 * i + j];
    for (int i = 0; i < nt; ++i)
        for (int j = 0; j < 3; ++j) Fm(i, j) = F[3 * i + j];
    Vec3 mn, mx;
    for (int j = 0; j < 3; ++j) {
        mn[j] = Vm.col(j).minCoeff();
        mx[j] = Vm.col(j).maxCoeff();
    }
    std::streambuf* old = std::cout.rdbuf(nullptr);
    std::vector<Vec3> pts = GeometryLoading::GeneratePointCloudFromWatertightTriangleMesh(Vm, Fm, mn, mx, (Real)dx);
    std::cout.rdbuf(old);
    const int k = (int)std::min<size_t>(pts.size(), (size_t)cap);
    for (int i = 0; i < k; ++i) put(pts[i], out + 3 * i);
    return (int)pts.size();
}

}  // extern "C"
