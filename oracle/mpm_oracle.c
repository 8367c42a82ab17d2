/*
 * mpm_oracle.c -- FP64 CPU restatement of the DiffMPMLib3D hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * `--impl reference` leg may load it.  The product (libmpm.so and the
 * diffmpm_bindings package) never links or calls it.
 *
 * It restates, in double precision, the reference algorithm for
 *   - the cubic B-spline kernel            DiffMPMLib3D/Interpolation.h:5-30
 *   - FCR stress P(F)                       DiffMPMLib3D/Elasticity.cpp:45-55
 *   - FCR Hessian-vector product            DiffMPMLib3D/Elasticity.cpp:12-31,57-117
 *   - one forward step                      DiffMPMLib3D/ForwardSimulation.cpp:16-185
 *   - one adjoint step                      DiffMPMLib3D/BackPropagation.cpp:9-144
 *   - the end-layer mass loss               DiffMPMLib3D/CompGraph.cpp:42-129
 *   - Adam / gradient norm                  DiffMPMLib3D/PointCloud.cpp:24-35,83-147
 *   - particle volumes / P2G utility        DiffMPMLib3D/ForwardSimulation.cpp:234-271
 *   - Lame parameters                       DiffMPMLib3D/Elasticity.cpp:149-153
 * plus an "exact" adjoint (the true derivative of the forward step) and the
 * optional quadratic-kernel / Neo-Hookean variants.
 *
 * The polar decomposition is computed here with a scaled Newton iteration
 * (Higham 1986, "Computing the polar decomposition -- with applications")
 * for det F > 0 and with a Jacobi eigen-decomposition of F^T F followed by a
 * rotation-variant SVD otherwise.  For non-singular F the rotation factor is
 * unique, so this agrees with the implicit-QR SVD the reference calls
 * (include/qrsvd/ImplicitQRSVD.h:401-450) to rounding.
 *
 * Array layout: vectors are (N,3) row-major, matrices (N,3,3) row-major,
 * grid node (i,j,k) lives at i*dy*dz + j*dz + k (Grid.h:89-94).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int dims[3];
    double dx;
    double min[3];
} orc_grid;

typedef struct {
    double dt, drag, smoothing;
    double f_ext[3];
    double bulk_visc;   /* 0.25 in the reference (ForwardSimulation.cpp:13)   */
    double j_min;       /* 0.60 trust-region floor; <= 0 disables it          */
    int exact;          /* 0: term-for-term BackPropagation.cpp; 1: true adjoint */
    int kernel;         /* 0: cubic B-spline (reference); 1: quadratic        */
    int material;       /* 0: fixed-corotated (reference); 1: Neo-Hookean     */
} orc_params;

/* ------------------------------------------------------------------ 3x3 */

static double det3(const double *A)
{
    return A[0] * (A[4] * A[8] - A[5] * A[7])
         - A[1] * (A[3] * A[8] - A[5] * A[6])
         + A[2] * (A[3] * A[7] - A[4] * A[6]);
}

/* cofactor matrix: cof(A) = det(A) * A^{-T} */
static void cof3(const double *A, double *c)
{
    c[0] = A[4] * A[8] - A[5] * A[7];
    c[1] = A[5] * A[6] - A[3] * A[8];
    c[2] = A[3] * A[7] - A[4] * A[6];
    c[3] = A[2] * A[7] - A[1] * A[8];
    c[4] = A[0] * A[8] - A[2] * A[6];
    c[5] = A[1] * A[6] - A[0] * A[7];
    c[6] = A[1] * A[5] - A[2] * A[4];
    c[7] = A[2] * A[3] - A[0] * A[5];
    c[8] = A[0] * A[4] - A[1] * A[3];
}

/* A^{-T}; returns det(A) */
static double invT3(const double *A, double *out)
{
    double c[9];
    cof3(A, c);
    double d = A[0] * c[0] + A[1] * c[1] + A[2] * c[2];
    for (int i = 0; i < 9; ++i) out[i] = c[i] / d;
    return d;
}

static void mul3(const double *A, const double *B, double *C)
{
    double t[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            t[r * 3 + c] = A[r * 3 + 0] * B[0 * 3 + c] + A[r * 3 + 1] * B[1 * 3 + c] + A[r * 3 + 2] * B[2 * 3 + c];
    memcpy(C, t, sizeof t);
}

/* A^T B */
static void mulTN3(const double *A, const double *B, double *C)
{
    double t[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            t[r * 3 + c] = A[0 * 3 + r] * B[0 * 3 + c] + A[1 * 3 + r] * B[1 * 3 + c] + A[2 * 3 + r] * B[2 * 3 + c];
    memcpy(C, t, sizeof t);
}

/* A B^T */
static void mulNT3(const double *A, const double *B, double *C)
{
    double t[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            t[r * 3 + c] = A[r * 3 + 0] * B[c * 3 + 0] + A[r * 3 + 1] * B[c * 3 + 1] + A[r * 3 + 2] * B[c * 3 + 2];
    memcpy(C, t, sizeof t);
}

static double ddot9(const double *A, const double *B)
{
    double s = 0;
    for (int i = 0; i < 9; ++i) s += A[i] * B[i];
    return s;
}

static double frob(const double *A) { return sqrt(ddot9(A, A)); }

/* ------------------------------------------------------- polar / SVD */

/* cyclic Jacobi eigen-decomposition of a symmetric 3x3 matrix A:
 * A = V diag(w) V^T, V columns are eigenvectors. */
static void sym_eig3(const double *Ain, double *w, double *V)
{
    double A[9];
    memcpy(A, Ain, sizeof A);
    for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
        double diag = A[0] * A[0] + A[4] * A[4] + A[8] * A[8];
        if (off <= 1e-300 || off <= 1e-34 * diag) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                double apq = A[p * 3 + q];
                if (apq == 0.0) continue;
                double app = A[p * 3 + p], aqq = A[q * 3 + q];
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                A[p * 3 + p] = app - t * apq;
                A[q * 3 + q] = aqq + t * apq;
                A[p * 3 + q] = A[q * 3 + p] = 0.0;
                int r = 3 - p - q;
                double arp = A[r * 3 + p], arq = A[r * 3 + q];
                A[r * 3 + p] = A[p * 3 + r] = c * arp - s * arq;
                A[r * 3 + q] = A[q * 3 + r] = s * arp + c * arq;
                for (int k = 0; k < 3; ++k) {
                    double vkp = V[k * 3 + p], vkq = V[k * 3 + q];
                    V[k * 3 + p] = c * vkp - s * vkq;
                    V[k * 3 + q] = s * vkp + c * vkq;
                }
            }
    }
    w[0] = A[0]; w[1] = A[4]; w[2] = A[8];
}

/* rotation-variant polar factor through an SVD: R = U V^T with det R = +1,
 * the sign of det F carried by the smallest singular value. */
static void polar_svd(const double *F, double *R)
{
    double FtF[9], w[3], V[9];
    mulTN3(F, F, FtF);
    sym_eig3(FtF, w, V);
    /* sort eigenpairs descending */
    int ord[3] = {0, 1, 2};
    for (int a = 0; a < 3; ++a)
        for (int b = a + 1; b < 3; ++b)
            if (w[ord[b]] > w[ord[a]]) { int t = ord[a]; ord[a] = ord[b]; ord[b] = t; }
    double Vs[9];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) Vs[r * 3 + c] = V[r * 3 + ord[c]];
    if (det3(Vs) < 0) for (int r = 0; r < 3; ++r) Vs[r * 3 + 2] = -Vs[r * 3 + 2];
    double u[3][3];
    for (int c = 0; c < 2; ++c)
        for (int r = 0; r < 3; ++r)
            u[c][r] = F[r * 3 + 0] * Vs[0 * 3 + c] + F[r * 3 + 1] * Vs[1 * 3 + c] + F[r * 3 + 2] * Vs[2 * 3 + c];
    double n1 = sqrt(u[0][0] * u[0][0] + u[0][1] * u[0][1] + u[0][2] * u[0][2]);
    if (n1 > 1e-300) { for (int r = 0; r < 3; ++r) u[0][r] /= n1; }
    else { u[0][0] = 1; u[0][1] = 0; u[0][2] = 0; }
    double d = u[0][0] * u[1][0] + u[0][1] * u[1][1] + u[0][2] * u[1][2];
    for (int r = 0; r < 3; ++r) u[1][r] -= d * u[0][r];
    double n2 = sqrt(u[1][0] * u[1][0] + u[1][1] * u[1][1] + u[1][2] * u[1][2]);
    if (n2 > 1e-14 * (n1 > 1e-300 ? n1 : 1.0)) { for (int r = 0; r < 3; ++r) u[1][r] /= n2; }
    else {
        /* any unit vector orthogonal to u0 */
        double e[3] = {0, 0, 0};
        int k = (fabs(u[0][0]) < fabs(u[0][1])) ? (fabs(u[0][0]) < fabs(u[0][2]) ? 0 : 2) : (fabs(u[0][1]) < fabs(u[0][2]) ? 1 : 2);
        e[k] = 1;
        double dd = e[0] * u[0][0] + e[1] * u[0][1] + e[2] * u[0][2];
        for (int r = 0; r < 3; ++r) u[1][r] = e[r] - dd * u[0][r];
        double nn = sqrt(u[1][0] * u[1][0] + u[1][1] * u[1][1] + u[1][2] * u[1][2]);
        for (int r = 0; r < 3; ++r) u[1][r] /= nn;
    }
    u[2][0] = u[0][1] * u[1][2] - u[0][2] * u[1][1];
    u[2][1] = u[0][2] * u[1][0] - u[0][0] * u[1][2];
    u[2][2] = u[0][0] * u[1][1] - u[0][1] * u[1][0];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            R[r * 3 + c] = u[0][r] * Vs[c * 3 + 0] + u[1][r] * Vs[c * 3 + 1] + u[2][r] * Vs[c * 3 + 2];
}

/* F = R S, R rotation, S symmetric */
void orc_polar(const double *F, double *R, double *S)
{
    double J = det3(F), nF = frob(F);
    int ok = isfinite(J) && nF > 0 && J > 1e-8 * nF * nF * nF;
    if (ok) {
        double X[9], Y[9], Xit[9];
        memcpy(X, F, sizeof X);
        int scale = 1;
        for (int it = 0; it < 100; ++it) {
            invT3(X, Xit);
            double g = 1.0;
            if (scale) g = sqrt(frob(Xit) / frob(X));
            for (int i = 0; i < 9; ++i) Y[i] = 0.5 * (g * X[i] + Xit[i] / g);
            double diff = 0;
            for (int i = 0; i < 9; ++i) diff += (Y[i] - X[i]) * (Y[i] - X[i]);
            diff = sqrt(diff);
            memcpy(X, Y, sizeof X);
            if (diff < 1e-2) scale = 0;
            if (diff <= 4e-16 * frob(Y)) break;
        }
        memcpy(R, X, sizeof X);
    } else {
        polar_svd(F, R);
    }
    double RtF[9];
    mulTN3(R, F, RtF);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) S[r * 3 + c] = 0.5 * (RtF[r * 3 + c] + RtF[c * 3 + r]);
}

/* --------------------------------------------------------- constitutive */

/* P(F) -- Elasticity.cpp:45-55 (FCR); Neo-Hookean optional. */
void orc_pk(int material, const double *F, double lam, double mu, double *P)
{
    double Fit[9];
    double Jraw = invT3(F, Fit);
    double J = Jraw > 1e-6 ? Jraw : 1e-6;
    if (material == 0) {
        double R[9], S[9];
        orc_polar(F, R, S);
        for (int i = 0; i < 9; ++i) P[i] = 2.0 * mu * (F[i] - R[i]) + lam * (J - 1.0) * J * Fit[i];
    } else {
        double lj = log(J);
        for (int i = 0; i < 9; ++i) P[i] = mu * (F[i] - Fit[i]) + lam * lj * Fit[i];
    }
}

/* Fit X^T Fit */
static void sandwichT(const double *Fit, const double *X, double *out)
{
    double t[9];
    mulNT3(Fit, X, t);    /* Fit X^T */
    mul3(t, Fit, out);    /* Fit X^T Fit */
}

/* -2 mu dR[dF] for the polar rotation, Elasticity.cpp:87-115 */
static void drot_term(const double *R, const double *S, const double *dF, double mu, double *out)
{
    double A[9] = {S[4] + S[8], -S[1], -S[2],
                   -S[1], S[0] + S[8], -S[5],
                   -S[2], -S[5], S[0] + S[4]};
    if (fabs(det3(A)) < 1e-6)
        for (int i = 0; i < 3; ++i) A[i * 4] += 1e-4;
    double t[9];
    mulTN3(R, dF, t);
    double b[3] = {t[7] - t[5], t[2] - t[6], t[3] - t[1]};
    double Ait[9];
    invT3(A, Ait);  /* A^{-T}; A is symmetric so A^{-1} = A^{-T} */
    double w[3];
    for (int r = 0; r < 3; ++r) w[r] = Ait[r * 3 + 0] * b[0] + Ait[r * 3 + 1] * b[1] + Ait[r * 3 + 2] * b[2];
    double W[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
    double dR[9];
    mul3(R, W, dR);
    for (int i = 0; i < 9; ++i) out[i] -= 2.0 * mu * dR[i];
}

/* Vector-Jacobian product of P(F) applied to G (= dL/dP): returns dL/dF.
 * exact == 0 reproduces d2_FCE_psi_dF2_mult_by_dF (Elasticity.cpp:57-117),
 * including its mix of clamped and unclamped J. */
void orc_pk_vjp(int material, int exact, const double *F, double lam, double mu, const double *G, double *out)
{
    double Fit[9];
    double Jraw = invT3(F, Fit);
    double J = Jraw > 1e-6 ? Jraw : 1e-6;
    double fg = ddot9(Fit, G);
    double sw[9];
    sandwichT(Fit, G, sw);
    if (material == 0) {
        double R[9], S[9];
        orc_polar(F, R, S);
        for (int i = 0; i < 9; ++i) out[i] = 2.0 * mu * G[i];
        if (!exact || Jraw > 1e-6) {
            /* lam*J*Fit*<J*Fit,G> + lam*(J-1)*Jraw*(<Fit,G>Fit - Fit G^T Fit) */
            for (int i = 0; i < 9; ++i)
                out[i] += lam * J * J * fg * Fit[i] + lam * (J - 1.0) * Jraw * (fg * Fit[i] - sw[i]);
        } else {
            /* J clamped to a constant: only Fit varies */
            for (int i = 0; i < 9; ++i) out[i] += -lam * (J - 1.0) * J * sw[i];
        }
        drot_term(R, S, G, mu, out);
    } else {
        double lj = log(J);
        for (int i = 0; i < 9; ++i) {
            out[i] = mu * G[i] + (mu - lam * lj) * sw[i];
            if (Jraw > 1e-6) out[i] += lam * fg * Fit[i];
        }
    }
}

void orc_lame(double E, double nu, double *lam, double *mu)
{
    *lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    *mu = E / (2.0 + 2.0 * nu);
}

/* ------------------------------------------------------------- kernel */

static double bspline(int kernel, double x, double *slope)
{
    double ax = fabs(x);
    if (kernel == 0) { /* cubic, Interpolation.h:5-30 */
        if (ax < 1.0) { *slope = 1.5 * x * ax - 2.0 * x; return 0.5 * ax * ax * ax - ax * ax + 2.0 / 3.0; }
        if (ax < 2.0) { *slope = -x * ax / 2.0 + 2.0 * x - 2.0 * x / ax; return (2.0 - ax) * (2.0 - ax) * (2.0 - ax) / 6.0; }
        *slope = 0; return 0;
    }
    if (ax < 0.5) { *slope = -2.0 * x; return 0.75 - x * x; }
    if (ax < 1.5) { *slope = (ax - 1.5) * (x > 0 ? 1.0 : -1.0); return 0.5 * (1.5 - ax) * (1.5 - ax); }
    *slope = 0; return 0;
}

#define KMAX 4

typedef struct {
    int K;
    int base[3];
    double w[3][KMAX];   /* N(dg/dx) per axis        */
    double s[3][KMAX];   /* N'(dg/dx) per axis       */
    double g[3][KMAX];   /* dg = node position - x   */
} stencil_t;

/* stencil of particle x: ForwardSimulation.cpp:28-54 (base index), Grid.cpp:7-26 (node x) */
static void make_stencil(const orc_grid *G, int kernel, const double *x, stencil_t *st)
{
    st->K = kernel == 0 ? 4 : 3;
    for (int a = 0; a < 3; ++a) {
        double rel = (x[a] - G->min[a]) / G->dx;
        st->base[a] = kernel == 0 ? (int)floor(rel) - 1 : (int)floor(rel - 0.5);
        for (int o = 0; o < st->K; ++o) {
            double node = G->min[a] + (double)(st->base[a] + o) * G->dx;
            double dg = node - x[a];
            st->g[a][o] = dg;
            st->w[a][o] = bspline(kernel, dg / G->dx, &st->s[a][o]);
        }
    }
}

static double apic_c0(int kernel, double dx) { return (kernel == 0 ? 3.0 : 4.0) / (dx * dx); }

static long long n_nodes(const orc_grid *G) { return (long long)G->dims[0] * G->dims[1] * G->dims[2]; }

#define FOR_STENCIL(G, st, ...)                                                        \
    for (int a_ = 0; a_ < (st).K; ++a_) {                                                 \
        int i_ = (st).base[0] + a_;                                                       \
        if (i_ < 0 || i_ >= (G)->dims[0]) continue;                                       \
        for (int b_ = 0; b_ < (st).K; ++b_) {                                             \
            int j_ = (st).base[1] + b_;                                                   \
            if (j_ < 0 || j_ >= (G)->dims[1]) continue;                                   \
            for (int c_ = 0; c_ < (st).K; ++c_) {                                         \
                int k_ = (st).base[2] + c_;                                               \
                if (k_ < 0 || k_ >= (G)->dims[2]) continue;                               \
                long long node_ = ((long long)i_ * (G)->dims[1] + j_) * (G)->dims[2] + k_;  \
                double w_ = (st).w[0][a_] * (st).w[1][b_] * (st).w[2][c_];                \
                double dg_[3] = {(st).g[0][a_], (st).g[1][b_], (st).g[2][c_]};            \
                (void)w_;                                                                 \
                (void)dg_;                                                                \
                __VA_ARGS__                                                               \
            }                                                                             \
        }                                                                                 \
    }

/* dw/dx_p = -(1/dx) (N'x Ny Nz, Nx N'y Nz, Nx Ny N'z), BackPropagation.cpp:95-104 */
#define GRADW(G, st, gw)                                                                   \
    double gw[3] = {-(st).s[0][a_] * (st).w[1][b_] * (st).w[2][c_] / (G)->dx,               \
                    -(st).w[0][a_] * (st).s[1][b_] * (st).w[2][c_] / (G)->dx,               \
                    -(st).w[0][a_] * (st).w[1][b_] * (st).s[2][c_] / (G)->dx};

static void atomic_add(double *p, double v)
{
#pragma omp atomic
    *p += v;
}

/* ---------------------------------------------------------------- P2G */

/* P2G of one particle set, ForwardSimulation.cpp:26-80.  Accumulates into gm/gp
 * (no reset).  P may be NULL when dt == 0 (the stress term vanishes). */
static void p2g(const orc_grid *G, const orc_params *prm, int n,
                const double *x, const double *v, const double *C, const double *F, const double *dFc,
                const double *m, const double *vol, const double *P, double *gm, double *gp)
{
    double C0 = apic_c0(prm->kernel, G->dx);
#pragma omp parallel for schedule(static)
    for (int p = 0; p < n; ++p) {
        stencil_t st;
        make_stencil(G, prm->kernel, x + 3 * p, &st);
        double A[9], mv[3];
        const double *Cp = C + 9 * p;
        double trC = Cp[0] + Cp[4] + Cp[8];
        if (P != NULL && prm->dt != 0.0) {
            double Ft[9], PFt[9];
            for (int i = 0; i < 9; ++i) Ft[i] = F[9 * p + i] + (dFc ? dFc[9 * p + i] : 0.0);
            mulNT3(P + 9 * p, Ft, PFt);
            for (int i = 0; i < 9; ++i) PFt[i] += (i % 4 == 0) ? prm->bulk_visc * trC : 0.0;
            for (int i = 0; i < 9; ++i) A[i] = -C0 * prm->dt * vol[p] * PFt[i] + m[p] * Cp[i];
        } else {
            /* dt == 0: stress and viscosity terms carry a factor dt */
            for (int i = 0; i < 9; ++i) A[i] = m[p] * Cp[i];
        }
        for (int a = 0; a < 3; ++a) mv[a] = m[p] * v[3 * p + a] * (1.0 - prm->dt * prm->drag);
        FOR_STENCIL(G, st, {
            atomic_add(&gm[node_], w_ * m[p]);
            if (gp) {
                for (int r = 0; r < 3; ++r)
                    atomic_add(&gp[3 * node_ + r],
                               w_ * (mv[r] + A[r * 3 + 0] * dg_[0] + A[r * 3 + 1] * dg_[1] + A[r * 3 + 2] * dg_[2]));
            }
        })
    }
}

/* --------------------------------------------------------- forward step */

/* One ForwardTimeStep (ForwardSimulation.cpp:159-185):
 * P_op_1, G_Reset, P2G, mass clamp, G_op, G2P, P_op_2.
 * gm/gp/gv receive the step's grid; trust_out (optional) the trust-region
 * scale applied to C (1 where inactive). */
int orc_forward_step(const orc_grid *G, const orc_params *prm, int n,
                     const double *x, const double *v, const double *C, const double *F, const double *dFc,
                     const double *m, const double *vol, const double *lam, const double *mu,
                     double *x1, double *v1, double *C1, double *F1,
                     double *gm, double *gp, double *gv, double *trust_out)
{
    long long nn = n_nodes(G);
    double *P = (double *)malloc(sizeof(double) * 9 * (size_t)(n > 0 ? n : 1));
    if (!P) return 3;
    /* P_op_1 */
#pragma omp parallel for schedule(static)
    for (int p = 0; p < n; ++p) {
        double Ft[9];
        for (int i = 0; i < 9; ++i) Ft[i] = F[9 * p + i] + (dFc ? dFc[9 * p + i] : 0.0);
        orc_pk(prm->material, Ft, lam[p], mu[p], P + 9 * p);
    }
    /* G_Reset */
    memset(gm, 0, sizeof(double) * nn);
    memset(gp, 0, sizeof(double) * 3 * nn);
    memset(gv, 0, sizeof(double) * 3 * nn);
    p2g(G, prm, n, x, v, C, F, dFc, m, vol, P, gm, gp);
    free(P);
    /* clamp + G_op (ForwardSimulation.cpp:82-87,165-170) */
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nn; ++i) {
        if (gm[i] < 0) gm[i] = 0;
        if (gm[i] > 1e-12)
            for (int a = 0; a < 3; ++a) gv[3 * i + a] = gp[3 * i + a] / gm[i] + prm->dt * prm->f_ext[a];
    }
    /* G2P + P_op_2 (ForwardSimulation.cpp:89-157) */
    double C0 = apic_c0(prm->kernel, G->dx);
#pragma omp parallel for schedule(static)
    for (int p = 0; p < n; ++p) {
        stencil_t st;
        make_stencil(G, prm->kernel, x + 3 * p, &st);
        double vn[3] = {0, 0, 0}, Cn[9] = {0};
        FOR_STENCIL(G, st, {
            const double *vi = gv + 3 * node_;
            for (int r = 0; r < 3; ++r) {
                vn[r] += w_ * vi[r];
                for (int c = 0; c < 3; ++c) Cn[r * 3 + c] += C0 * w_ * vi[r] * dg_[c];
            }
        })
        double Ft[9];
        for (int i = 0; i < 9; ++i) Ft[i] = F[9 * p + i] + (dFc ? dFc[9 * p + i] : 0.0);
        double s_tr = 1.0;
        if (prm->j_min > 0) {
            double J0 = det3(Ft);
            if (J0 < 1e-6) J0 = 1e-6;
            double trC = Cn[0] + Cn[4] + Cn[8];
            if (trC < 0) {
                double denom = prm->dt * trC;
                double s = (prm->j_min / J0 - 1.0) / (denom < -1e-6 ? denom : -1e-6);
                if (s < 1.0) {
                    s_tr = s < 0 ? 0 : s;
                    for (int i = 0; i < 9; ++i) Cn[i] *= s_tr;
                }
            }
        }
        double IdtC[9], Fn[9];
        for (int i = 0; i < 9; ++i) IdtC[i] = (i % 4 == 0 ? 1.0 : 0.0) + prm->dt * Cn[i];
        mul3(IdtC, Ft, Fn);
        for (int i = 0; i < 9; ++i)
            F1[9 * p + i] = Fn[i] * (1.0 - prm->smoothing) + F[9 * p + i] * prm->smoothing;
        for (int a = 0; a < 3; ++a) {
            v1[3 * p + a] = vn[a];
            x1[3 * p + a] = x[3 * p + a] + prm->dt * vn[a];
        }
        memcpy(C1 + 9 * p, Cn, sizeof Cn);
        if (trust_out) trust_out[p] = s_tr;
    }
    return 0;
}

/* -------------------------------------------------------- adjoint step */

/* One Back_Timestep (BackPropagation.cpp:9-144).
 * Inputs: layer n state, layer n+1 C (C1) and gradients (gx1,gv1,gF1,gC1),
 * grid mass/velocity of step n (gm, gv), trust scale of step n (exact only).
 * Outputs (overwritten): layer n gradients gx,gv,gF,gC.  Optional outputs:
 * gFt = dL/d(F+dFc) (the control gradient, exact mode), glam/gmu (+=). */
int orc_backward_step(const orc_grid *G, const orc_params *prm, int n,
                      const double *x, const double *v, const double *C, const double *F, const double *dFc,
                      const double *m, const double *vol, const double *lam, const double *mu,
                      const double *C1, const double *trust,
                      const double *gm, const double *gv_node,
                      const double *gx1, const double *gv1, const double *gF1, const double *gC1,
                      double *gx, double *gv, double *gF, double *gC,
                      double *gFt_out, double *glam, double *gmu)
{
    long long nn = n_nodes(G);
    double C0 = apic_c0(prm->kernel, G->dx);
    double dt = prm->dt, s = prm->smoothing;
    int exact = prm->exact;
    double *vbar = (double *)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    double *Cbar = (double *)malloc(sizeof(double) * 9 * (size_t)(n > 0 ? n : 1));
    double *Fpart = (double *)malloc(sizeof(double) * 9 * (size_t)(n > 0 ? n : 1));
    double *nd = (double *)calloc((size_t)nn * 4, sizeof(double)); /* dLdv -> (dLdp, dLdm) */
    if (!vbar || !Cbar || !Fpart || !nd) { free(vbar); free(Cbar); free(Fpart); free(nd); return 3; }

    /* P_op_2^T (BackPropagation.cpp:22-32) */
#pragma omp parallel for schedule(static)
    for (int p = 0; p < n; ++p) {
        const double *g = gF1 + 9 * p;
        double Ft[9], IdtC[9], t[9];
        for (int i = 0; i < 9; ++i) Ft[i] = F[9 * p + i] + (dFc ? dFc[9 * p + i] : 0.0);
        for (int i = 0; i < 9; ++i) IdtC[i] = (i % 4 == 0 ? 1.0 : 0.0) + dt * C1[9 * p + i];
        mulTN3(IdtC, g, t);
        double gFt[9];
        for (int i = 0; i < 9; ++i) gFt[i] = (1.0 - s) * t[i];
        for (int a = 0; a < 3; ++a) vbar[3 * p + a] = dt * gx1[3 * p + a] + gv1[3 * p + a];
        double gFtT[9];
        mulNT3(g, Ft, gFtT);  /* g Ft^T */
        double cb[9];
        for (int i = 0; i < 9; ++i) cb[i] = (exact ? (1.0 - s) : 1.0) * dt * gFtT[i] + gC1[9 * p + i];
        if (exact && prm->j_min > 0) {
            double st = trust ? trust[p] : 1.0;
            if (st <= 0.0) {
                for (int i = 0; i < 9; ++i) cb[i] = 0.0;
            } else if (st < 1.0) {
                double Cp[9];
                for (int i = 0; i < 9; ++i) Cp[i] = C1[9 * p + i] / st;
                double trCp = Cp[0] + Cp[4] + Cp[8];
                double denom = dt * trCp;
                double q = ddot9(cb, Cp);
                double dsdtr = denom < -1e-6 ? -st / trCp : 0.0;
                double Fit[9];
                double J0 = invT3(Ft, Fit);
                double dsdJ0 = J0 > 1e-6 ? -prm->j_min / (J0 * J0 * (denom < -1e-6 ? denom : -1e-6)) : 0.0;
                for (int i = 0; i < 9; ++i) {
                    cb[i] = st * cb[i] + ((i % 4 == 0) ? q * dsdtr : 0.0);
                    gFt[i] += q * dsdJ0 * J0 * Fit[i];
                }
            }
        }
        memcpy(Cbar + 9 * p, cb, sizeof cb);
        if (exact) memcpy(Fpart + 9 * p, gFt, sizeof gFt);
        else for (int i = 0; i < 9; ++i) Fpart[9 * p + i] = gFt[i] + s * g[i];
    }

    /* G2P^T scatter (BackPropagation.cpp:36-55) */
#pragma omp parallel for schedule(static)
    for (int p = 0; p < n; ++p) {
        stencil_t st;
        make_stencil(G, prm->kernel, x + 3 * p, &st);
        const double *vb = vbar + 3 * p, *cb = Cbar + 9 * p;
        FOR_STENCIL(G, st, {
            for (int r = 0; r < 3; ++r)
                atomic_add(&nd[4 * node_ + r],
                           w_ * vb[r] + C0 * w_ * (cb[r * 3 + 0] * dg_[0] + cb[r * 3 + 1] * dg_[1] + cb[r * 3 + 2] * dg_[2]));
        })
    }

    /* G_op^T (BackPropagation.cpp:59-72) */
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nn; ++i) {
        double mi = gm[i];
        double *d = nd + 4 * i;
        if (fabs(mi) > 1e-12) {
            double vv[3];
            for (int a = 0; a < 3; ++a) vv[a] = gv_node[3 * i + a] - (exact ? dt * prm->f_ext[a] : 0.0);
            double dm = -(vv[0] * d[0] + vv[1] * d[1] + vv[2] * d[2]) / mi;
            for (int a = 0; a < 3; ++a) d[a] = d[a] / mi;
            d[3] = dm;
        } else {
            d[0] = d[1] = d[2] = d[3] = 0.0;
        }
    }

    /* P2G^T + P_op_1^T (BackPropagation.cpp:76-143) */
#pragma omp parallel for schedule(static)
    for (int p = 0; p < n; ++p) {
        stencil_t st;
        make_stencil(G, prm->kernel, x + 3 * p, &st);
        double Ft[9], P[9];
        for (int i = 0; i < 9; ++i) Ft[i] = F[9 * p + i] + (dFc ? dFc[9 * p + i] : 0.0);
        orc_pk(prm->material, Ft, lam[p], mu[p], P);
        const double *Cp = C + 9 * p;
        double trC = Cp[0] + Cp[4] + Cp[8];
        double PFt[9], A[9];
        mulNT3(P, Ft, PFt);
        for (int i = 0; i < 9; ++i)
            A[i] = -C0 * dt * vol[p] * (PFt[i] + ((i % 4 == 0) ? prm->bulk_visc * trC : 0.0)) + m[p] * Cp[i];
        double mvv[3];
        for (int a = 0; a < 3; ++a) mvv[a] = m[p] * v[3 * p + a] * (exact ? (1.0 - dt * prm->drag) : 1.0);
        const double *vb = vbar + 3 * p, *cb = Cbar + 9 * p;
        double M1[9] = {0}, ax[3] = {0, 0, 0}, bp[3] = {0, 0, 0}, bv[3] = {0, 0, 0};
        FOR_STENCIL(G, st, {
            GRADW(G, st, gw)
            const double *d = nd + 4 * node_;
            const double *vi = gv_node + 3 * node_;
            double Adg[3], cdg[3];
            for (int r = 0; r < 3; ++r) {
                Adg[r] = A[r * 3 + 0] * dg_[0] + A[r * 3 + 1] * dg_[1] + A[r * 3 + 2] * dg_[2];
                cdg[r] = cb[r * 3 + 0] * dg_[0] + cb[r * 3 + 1] * dg_[1] + cb[r * 3 + 2] * dg_[2];
            }
            double sig = m[p] * d[3]
                       + (mvv[0] + Adg[0]) * d[0] + (mvv[1] + Adg[1]) * d[1] + (mvv[2] + Adg[2]) * d[2]
                       + vi[0] * vb[0] + vi[1] * vb[1] + vi[2] * vb[2]
                       + C0 * (vi[0] * cdg[0] + vi[1] * cdg[1] + vi[2] * cdg[2]);
            for (int r = 0; r < 3; ++r) {
                ax[r] += sig * gw[r];
                bp[r] += w_ * d[r];
                bv[r] += w_ * vi[r];
                for (int c = 0; c < 3; ++c) M1[r * 3 + c] += w_ * d[r] * dg_[c];
            }
        })
        /* dL/dx: mass + momentum (stencil part) + v_next + C_next, then the
         * -w G^T dLdp and -w C0 dLdC_next^T v terms, and dLdx_{n+1}. */
        double AtB[3], CtV[3];
        for (int r = 0; r < 3; ++r) {
            AtB[r] = A[0 * 3 + r] * bp[0] + A[1 * 3 + r] * bp[1] + A[2 * 3 + r] * bp[2];
            CtV[r] = cb[0 * 3 + r] * bv[0] + cb[1 * 3 + r] * bv[1] + cb[2 * 3 + r] * bv[2];
        }
        for (int r = 0; r < 3; ++r) {
            gx[3 * p + r] = ax[r] - AtB[r] - C0 * CtV[r] + gx1[3 * p + r];
            gv[3 * p + r] = m[p] * (1.0 - dt * prm->drag) * bp[r];
        }
        /* dL/dC: m M1 + bulk viscosity */
        double k = -C0 * dt * vol[p] * prm->bulk_visc;
        double trM = M1[0] + M1[4] + M1[8];
        for (int i = 0; i < 9; ++i) {
            double add = 0.0;
            if (i % 4 == 0) add = exact ? k * trM : k * M1[i];
            gC[9 * p + i] = m[p] * M1[i] + add;
        }
        /* dL/dP = -C0 dt vol M1 Ft ; dL/dFt += -C0 dt vol M1^T P */
        double gP[9], t1[9], t2[9];
        mul3(M1, Ft, t1);
        mulTN3(M1, P, t2);
        double kk = -C0 * dt * vol[p];
        for (int i = 0; i < 9; ++i) gP[i] = kk * t1[i];
        double gFt[9], hv[9];
        orc_pk_vjp(prm->material, exact, Ft, lam[p], mu[p], gP, hv);
        for (int i = 0; i < 9; ++i) gFt[i] = Fpart[9 * p + i] + kk * t2[i] + hv[i];
        if (!exact) {
            /* BackPropagation.cpp:140 adds (I + dt C_{n+1})^T dLdF_{n+1} a second time */
            double IdtC[9], t[9];
            for (int i = 0; i < 9; ++i) IdtC[i] = (i % 4 == 0 ? 1.0 : 0.0) + dt * C1[9 * p + i];
            mulTN3(IdtC, gF1 + 9 * p, t);
            for (int i = 0; i < 9; ++i) gFt[i] += t[i];
            memcpy(gF + 9 * p, gFt, sizeof gFt);
            if (gFt_out) memcpy(gFt_out + 9 * p, gFt, sizeof gFt);
        } else {
            for (int i = 0; i < 9; ++i) gF[9 * p + i] = gFt[i] + s * gF1[9 * p + i];
            if (gFt_out) memcpy(gFt_out + 9 * p, gFt, sizeof gFt);
        }
        if (glam || gmu) {
            double Fit[9], R[9], S[9];
            double Jraw = invT3(Ft, Fit);
            double J = Jraw > 1e-6 ? Jraw : 1e-6;
            if (prm->material == 0) {
                orc_polar(Ft, R, S);
                double dmu = 0, dl = 0;
                for (int i = 0; i < 9; ++i) { dmu += gP[i] * 2.0 * (Ft[i] - R[i]); dl += gP[i] * (J - 1.0) * J * Fit[i]; }
                if (gmu) gmu[p] += dmu;
                if (glam) glam[p] += dl;
            } else {
                double dmu = 0, dl = 0;
                for (int i = 0; i < 9; ++i) { dmu += gP[i] * (Ft[i] - Fit[i]); dl += gP[i] * log(J) * Fit[i]; }
                if (gmu) gmu[p] += dmu;
                if (glam) glam[p] += dl;
            }
        }
    }
    free(vbar); free(Cbar); free(Fpart); free(nd);
    return 0;
}

/* ------------------------------------------------------------ mass loss */

/* EndLayerMassLoss (CompGraph.cpp:42-129).  Writes the grid mass of the last
 * layer into gm, dL/dm per node into dLdm, and dL/dx per particle into gx.
 * exact != 0 drops the x5 out-of-target factor and keeps the derivative of
 * the global mass scale s. */
double orc_mass_loss(const orc_grid *G, const orc_params *prm, int n,
                     const double *x, const double *m, const double *target_m,
                     double *gm, double *dLdm, double *gx)
{
    long long nn = n_nodes(G);
    const double eps = 1e-4, min_mass = 1e-3, pw = 1.0, pen_out = 5.0, eps_s = 1e-6;
    memset(gm, 0, sizeof(double) * nn);
    double *zero9 = NULL;
    (void)zero9;
    /* P2G with dt = drag = 0 (mass only matters) */
    orc_params q = *prm;
    q.dt = 0; q.drag = 0;
    double *zC = (double *)calloc((size_t)(n > 0 ? n : 1) * 9, sizeof(double));
    double *zv = (double *)calloc((size_t)(n > 0 ? n : 1) * 3, sizeof(double));
    p2g(G, &q, n, x, zv, zC, zC, NULL, m, m, NULL, gm, NULL);
    free(zC); free(zv);
    double sum_c = 0, sum_t = 0;
    for (long long i = 0; i < nn; ++i) { sum_c += gm[i]; sum_t += target_m[i]; }
    double sc = (sum_t + eps_s) / (sum_c + eps_s);
    double loss = 0, gc = 0;
#pragma omp parallel for reduction(+ : loss, gc) schedule(static)
    for (long long i = 0; i < nn; ++i) {
        double cms = sc * gm[i];
        double ld = log(cms + 1.0 + eps) - log(target_m[i] + 1.0 + eps);
        loss += 0.5 * ld * ld;
        double g = ld / (cms + 1.0 + eps);   /* dL_i/d(cms) */
        if (cms < min_mass) {
            double diff = min_mass - cms;
            loss += pw * diff * diff;
            g += -2.0 * pw * diff;
        }
        dLdm[i] = sc * g;
        gc += g * gm[i];
    }
    if (prm->exact) {
        double dsdc = -sc / (sum_c + eps_s);
        for (long long i = 0; i < nn; ++i) dLdm[i] += gc * dsdc;
    }
#pragma omp parallel for schedule(static)
    for (int p = 0; p < n; ++p) {
        stencil_t st;
        make_stencil(G, prm->kernel, x + 3 * p, &st);
        double a[3] = {0, 0, 0};
        FOR_STENCIL(G, st, {
            GRADW(G, st, gw)
            double pen = (prm->exact || target_m[node_] > 1e-12) ? 1.0 : pen_out;
            for (int r = 0; r < 3; ++r) a[r] += pen * m[p] * dLdm[node_] * gw[r];
        })
        for (int r = 0; r < 3; ++r) gx[3 * p + r] = a[r];
    }
    return loss;
}

/* ------------------------------------------------------------- volumes */

/* P2G(pc, grid, 0, 0) into an un-reset grid (bind.cpp:546-549). */
void orc_p2g_accumulate(const orc_grid *G, int kernel, int n,
                        const double *x, const double *v, const double *C, const double *m,
                        double *gm, double *gp)
{
    orc_params q;
    memset(&q, 0, sizeof q);
    q.kernel = kernel;
    p2g(G, &q, n, x, v, C, C, NULL, m, m, NULL, gm, gp);
}

/* CalculatePointCloudVolumes (ForwardSimulation.cpp:234-271) */
void orc_volumes(const orc_grid *G, int kernel, int n,
                 const double *x, const double *v, const double *C, const double *m,
                 double *gm, double *gp, double *vol)
{
    orc_p2g_accumulate(G, kernel, n, x, v, C, m, gm, gp);
    double cell = G->dx * G->dx * G->dx;
#pragma omp parallel for schedule(static)
    for (int p = 0; p < n; ++p) {
        stencil_t st;
        make_stencil(G, kernel, x + 3 * p, &st);
        double mg = 0;
        FOR_STENCIL(G, st, { mg += w_ * gm[node_]; })
        double rho = mg / (cell > 1e-12 ? cell : 1e-12);
        vol[p] = rho > FLT_EPSILON ? m[p] / rho : 0.0;
    }
}

/* ----------------------------------------------------------------- Adam */

double orc_grad_norm(int n, const double *g)
{
    double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long long i = 0; i < 9LL * n; ++i) s += g[i] * g[i];
    return sqrt(s);
}

/* Descend_Adam (PointCloud.cpp:83-147): AMSGrad, floored sqrt, per-particle
 * step cap and near-stationary EMA. */
void orc_adam(int n, const double *dLdF, double *dFc, double *mom, double *vec, double *vmax,
              double alpha, double gnorm, double beta1, double beta2, double eps, int timestep)
{
    const double vfloor = 1e-8, max_abs = 5e-3, max_rel = 5e-2, ema_k = 0.2, small_abs = 1e-4, small_rel = 1e-3;
    double inv_gn = 1.0 / (gnorm > 1e-12 ? gnorm : 1e-12);
    int t = timestep > 1 ? timestep : 1;
    double bc1 = 1.0 - pow(beta1, t), bc2 = 1.0 - pow(beta2, t);
#pragma omp parallel for schedule(static)
    for (int p = 0; p < n; ++p) {
        double step[9], xo[9];
        double sn = 0, xn = 0;
        for (int i = 0; i < 9; ++i) {
            int k = 9 * p + i;
            double g = dLdF[k] * inv_gn;
            mom[k] = beta1 * mom[k] + (1.0 - beta1) * g;
            vec[k] = beta2 * vec[k] + (1.0 - beta2) * g * g;
            double mh = mom[k] / bc1, vh = vec[k] / bc2;
            if (vh > vmax[k]) vmax[k] = vh;
            double den = sqrt(vmax[k]);
            if (den < vfloor) den = vfloor;
            step[i] = mh / (den + eps);
            sn += step[i] * step[i];
            xo[i] = dFc[k];
            xn += xo[i] * xo[i];
        }
        sn = sqrt(sn); xn = sqrt(xn);
        double cap = max_rel * (xn > 1.0 ? xn : 1.0);
        if (cap < max_abs) cap = max_abs;
        double scale = 1.0;
        if (sn > 0 && alpha * sn > cap) scale = cap / (alpha * sn);
        double small = small_rel * (xn > 1.0 ? xn : 1.0);
        if (small < small_abs) small = small_abs;
        int near = alpha * sn <= small;
        for (int i = 0; i < 9; ++i) {
            double nx = xo[i] - alpha * step[i] * scale;
            if (near) nx = xo[i] + ema_k * (nx - xo[i]);
            dFc[9 * p + i] = nx;
        }
    }
}

/* ------------------------------------------------------------- rollout */

/* Forward T steps from state 0 then the adjoint back to layer 0 with a
 * last-layer dL/dx seed; used to time the CPU baseline.  States for every
 * layer are kept (the reference keeps its full tape, CompGraph.cpp:30-40).
 * dFc0 (optional) is the control at layer 0.  Outputs the final x and the
 * layer-0 gradients.  Returns 0 on success. */
int orc_rollout(const orc_grid *G, const orc_params *prm, int n, int T,
                const double *x0, const double *v0, const double *F0, const double *dFc0,
                const double *m, const double *vol, const double *lam, const double *mu,
                const double *seed_gx, double *xT,
                double *gx0, double *gv0, double *gF0, double *gC0)
{
    size_t N3 = (size_t)n * 3, N9 = (size_t)n * 9;
    long long nn = n_nodes(G);
    double *X = (double *)malloc(sizeof(double) * N3 * (T + 1));
    double *V = (double *)malloc(sizeof(double) * N3 * (T + 1));
    double *Cs = (double *)calloc(N9 * (T + 1), sizeof(double));
    double *Fs = (double *)malloc(sizeof(double) * N9 * (T + 1));
    double *GM = (double *)malloc(sizeof(double) * nn * T);
    double *GV = (double *)malloc(sizeof(double) * 3 * nn * T);
    double *gp = (double *)malloc(sizeof(double) * 3 * nn);
    double *TR = (double *)malloc(sizeof(double) * (size_t)n * T);
    double *ga = (double *)calloc(N3 * 2 + N9 * 2, sizeof(double));
    double *gb = (double *)calloc(N3 * 2 + N9 * 2, sizeof(double));
    if (!X || !V || !Cs || !Fs || !GM || !GV || !gp || !TR || !ga || !gb) {
        free(X); free(V); free(Cs); free(Fs); free(GM); free(GV); free(gp); free(TR); free(ga); free(gb);
        return 3;
    }
    memcpy(X, x0, sizeof(double) * N3);
    memcpy(V, v0, sizeof(double) * N3);
    memcpy(Fs, F0, sizeof(double) * N9);
    for (int t = 0; t < T; ++t)
        orc_forward_step(G, prm, n, X + N3 * t, V + N3 * t, Cs + N9 * t, Fs + N9 * t, t == 0 ? dFc0 : NULL,
                         m, vol, lam, mu, X + N3 * (t + 1), V + N3 * (t + 1), Cs + N9 * (t + 1), Fs + N9 * (t + 1),
                         GM + nn * t, gp, GV + 3 * nn * t, TR + (size_t)n * t);
    memcpy(xT, X + N3 * T, sizeof(double) * N3);
    /* seed: dL/dx at the last layer, others zero */
    memcpy(ga, seed_gx, sizeof(double) * N3);
    for (int t = T - 1; t >= 0; --t) {
        double *gx1 = ga, *gv1 = ga + N3, *gF1 = ga + 2 * N3, *gC1 = ga + 2 * N3 + N9;
        double *gx = gb, *gv = gb + N3, *gF = gb + 2 * N3, *gC = gb + 2 * N3 + N9;
        orc_backward_step(G, prm, n, X + N3 * t, V + N3 * t, Cs + N9 * t, Fs + N9 * t, t == 0 ? dFc0 : NULL,
                          m, vol, lam, mu, Cs + N9 * (t + 1), TR + (size_t)n * t, GM + nn * t, GV + 3 * nn * t,
                          gx1, gv1, gF1, gC1, gx, gv, gF, gC, NULL, NULL, NULL);
        double *tmp = ga; ga = gb; gb = tmp;
    }
    memcpy(gx0, ga, sizeof(double) * N3);
    memcpy(gv0, ga + N3, sizeof(double) * N3);
    memcpy(gF0, ga + 2 * N3, sizeof(double) * N9);
    memcpy(gC0, ga + 2 * N3 + N9, sizeof(double) * N9);
    free(X); free(V); free(Cs); free(Fs); free(GM); free(GV); free(gp); free(TR); free(ga); free(gb);
    return 0;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Threads the OpenMP loops above use from now on (n >= 1); the CPU-baseline
 * legs time the reference algorithm on all host threads and on one, since
 * the reference's adjoint serialises its G2P transpose (omp critical,
 * BackPropagation.cpp:50-53) and runs no faster on many threads. */
void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n >= 1) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
