/* A plain C99 caller of libmpm.so (test infrastructure): the C ABI of
 * include/mpm.h used the way a host in another language would bind it, with
 * no Python in between.
 *
 *   c_caller host   host-only entry points (no GPU): defaults, the Lame
 *                   formula, argument checks and error messages
 *   c_caller sim    (GPU) a block of particles translating at constant
 *                   velocity with no stress, drag or external force:
 *                   forward T steps, then the exact adjoint of
 *                   L = mean_p x_T,p,x.  Checks x_T = x_0 + T dt v0 and
 *                   sum_p dL/dv0_p,x = T dt.
 * Prints "<mode> ok" and exits 0 on success. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mpm.h"

static int fail(const char* what, int rc)
{
    fprintf(stderr, "%s: status %d (%s)\n", what, rc, mpm_last_error());
    return 1;
}

#define CK(call)                                \
    do {                                        \
        const int rc_ = (call);                 \
        if (rc_ != MPM_OK) return fail(#call, rc_); \
    } while (0)

static int host_checks(void)
{
    mpm_params p;
    mpm_default_params(&p);
    if (fabs(p.dt - 1.0 / 120.0) > 1e-15 || p.drag != 0.5 || p.smoothing != 0.1) return fail("default params", -1);
    mpm_options o;
    mpm_default_options(&o);
    if (o.precision != MPM_FP32 || o.adjoint != MPM_ADJ_REFERENCE || o.checkpoint_every != 1)
        return fail("default options", -1);
    double lam = 0, mu = 0;
    CK(mpm_lame(1e4, 0.3, &lam, &mu));
    if (fabs(lam - 1e4 * 0.3 / (1.3 * 0.4)) > 1e-9 || fabs(mu - 1e4 / 2.6) > 1e-9) return fail("lame", -1);
    if (mpm_set_tile_nodes(-1) != MPM_ERR_ARG || strlen(mpm_last_error()) == 0) return fail("argument check", -1);
    if (mpm_compgraph_forward(NULL, 0, 0) != MPM_ERR_ARG) return fail("null graph", -1);
    printf("host ok (libmpm version %d)\n", mpm_version());
    return 0;
}

static int sim(void)
{
    enum { S = 8, N = S * S * S, T = 5 };
    const double dx = 1.0 / 32, dt = 1e-3, v0x = 0.1, rho = 60.0;
    const double pdx = 0.5 * dx, vol = pdx * pdx * pdx;
    double lam, mu;
    CK(mpm_lame(1e4, 0.3, &lam, &mu));
    double *x = malloc(sizeof(double) * 3 * N), *v = malloc(sizeof(double) * 3 * N),
           *F = malloc(sizeof(double) * 9 * N), *m = malloc(sizeof(double) * N), *vo = malloc(sizeof(double) * N),
           *la = malloc(sizeof(double) * N), *mm = malloc(sizeof(double) * N), *g = malloc(sizeof(double) * 3 * N);
    if (!x || !v || !F || !m || !vo || !la || !mm || !g) return fail("malloc", -1);
    for (int p = 0; p < N; ++p) {
        const int i = p / (S * S), j = (p / S) % S, k = p % S;
        x[3 * p] = 0.375 + (i + 0.5) * pdx;
        x[3 * p + 1] = 0.375 + (j + 0.5) * pdx;
        x[3 * p + 2] = 0.375 + (k + 0.5) * pdx;
        v[3 * p] = v0x;
        v[3 * p + 1] = v[3 * p + 2] = 0.0;
        for (int q = 0; q < 9; ++q) F[9 * p + q] = (q % 4 == 0) ? 1.0 : 0.0;
        m[p] = rho * vol;
        vo[p] = vol;
        la[p] = lam;
        mm[p] = mu;
    }
    mpm_pointcloud* pc = NULL;
    mpm_grid* grid = NULL;
    mpm_compgraph* cg = NULL;
    CK(mpm_pointcloud_create(N, MPM_FP32, &pc));
    CK(mpm_pointcloud_set(pc, MPM_FIELD_X, x, MPM_DTYPE_F64, 0));
    CK(mpm_pointcloud_set(pc, MPM_FIELD_V, v, MPM_DTYPE_F64, 0));
    CK(mpm_pointcloud_set(pc, MPM_FIELD_F, F, MPM_DTYPE_F64, 0));
    CK(mpm_pointcloud_set(pc, MPM_FIELD_M, m, MPM_DTYPE_F64, 0));
    CK(mpm_pointcloud_set(pc, MPM_FIELD_VOL, vo, MPM_DTYPE_F64, 0));
    CK(mpm_pointcloud_set(pc, MPM_FIELD_LAM, la, MPM_DTYPE_F64, 0));
    CK(mpm_pointcloud_set(pc, MPM_FIELD_MU, mm, MPM_DTYPE_F64, 0));
    const double gmin[3] = {0.0, 0.0, 0.0};
    CK(mpm_grid_create(33, 33, 33, dx, gmin, MPM_FP32, &grid));
    mpm_options o;
    mpm_default_options(&o);
    o.adjoint = MPM_ADJ_EXACT;
    CK(mpm_compgraph_create(pc, grid, grid, &o, &cg));
    mpm_params prm;
    mpm_default_params(&prm);
    prm.dt = dt;
    prm.drag = 0.0;
    prm.smoothing = 0.0;
    CK(mpm_compgraph_set_params(cg, &prm));
    CK(mpm_compgraph_set_up(cg, T + 1));
    CK(mpm_compgraph_forward(cg, 0, 0));
    mpm_pointcloud *last = NULL, *first = NULL;
    CK(mpm_compgraph_layer(cg, T, &last));
    CK(mpm_compgraph_layer(cg, 0, &first));
    CK(mpm_pointcloud_get(last, MPM_FIELD_X, g, MPM_DTYPE_F64, 0));
    double err = 0.0;
    for (int p = 0; p < N; ++p)
        for (int a = 0; a < 3; ++a) {
            const double want = x[3 * p + a] + (a == 0 ? T * dt * v0x : 0.0);
            const double e = fabs(g[3 * p + a] - want);
            if (!(e <= err)) err = e;  /* also catches NaN */
        }
    if (!(err < 1e-5)) {
        fprintf(stderr, "translation error %g\n", err);
        return 1;
    }
    /* L = mean over particles of x_T,x */
    for (int p = 0; p < N; ++p) {
        g[3 * p] = 1.0 / N;
        g[3 * p + 1] = g[3 * p + 2] = 0.0;
    }
    CK(mpm_pointcloud_set(last, MPM_FIELD_GRAD_X, g, MPM_DTYPE_F64, 0));
    CK(mpm_compgraph_backward(cg, 0));
    CK(mpm_pointcloud_get(first, MPM_FIELD_GRAD_V, g, MPM_DTYPE_F64, 0));
    double s = 0.0;
    for (int p = 0; p < N; ++p) s += g[3 * p];
    if (!(fabs(s - T * dt) < 1e-4 * T * dt)) {
        fprintf(stderr, "sum dL/dv0_x = %.9g, want %.9g\n", s, T * dt);
        return 1;
    }
    CK(mpm_pointcloud_release(first));
    CK(mpm_pointcloud_release(last));
    CK(mpm_compgraph_release(cg));
    CK(mpm_grid_release(grid));
    CK(mpm_pointcloud_release(pc));
    free(x); free(v); free(F); free(m); free(vo); free(la); free(mm); free(g);
    printf("sim ok (x_T error %.2e, sum dL/dv0_x %.9g)\n", err, s);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc > 1 && strcmp(argv[1], "sim") == 0) return sim();
    return host_checks();
}
