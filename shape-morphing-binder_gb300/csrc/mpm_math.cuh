// mpm_math.cuh -- per-particle device math for the MPM step and its adjoint.
//
// 3x3 matrices are row-major arrays of 9 scalars.  Everything is templated on
// the storage scalar R (float for the production path, double for the plain
// all-FP64 form).  The float path computes the polar decomposition in FP32
// (Newton-Schulz for a nearly orthogonal F, scaled Newton otherwise) and
// falls back to an FP64 Jacobi SVD when F is close to inversion (the FP64
// guard); J - 1 is formed from F - I so the
// volumetric stress does not lose digits to cancellation.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#define MPM_HD __host__ __device__ __forceinline__
#define MPM_D __device__ __forceinline__

namespace mpm {

// ---------------------------------------------------------------- 3x3 ops

template <typename R>
MPM_HD R det3(const R* A)
{
    return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
           A[2] * (A[3] * A[7] - A[4] * A[6]);
}

// cofactor matrix cof(A) = det(A) A^{-T}
template <typename R>
MPM_HD void cof3(const R* A, R* c)
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

template <typename R>
MPM_HD void mul3(const R* A, const R* B, R* C)  // C = A B
{
    R t[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) t[r * 3 + c] = A[r * 3] * B[c] + A[r * 3 + 1] * B[3 + c] + A[r * 3 + 2] * B[6 + c];
#pragma unroll
    for (int i = 0; i < 9; ++i) C[i] = t[i];
}

template <typename R>
MPM_HD void mulTN3(const R* A, const R* B, R* C)  // C = A^T B
{
    R t[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) t[r * 3 + c] = A[r] * B[c] + A[3 + r] * B[3 + c] + A[6 + r] * B[6 + c];
#pragma unroll
    for (int i = 0; i < 9; ++i) C[i] = t[i];
}

template <typename R>
MPM_HD void mulNT3(const R* A, const R* B, R* C)  // C = A B^T
{
    R t[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            t[r * 3 + c] = A[r * 3] * B[c * 3] + A[r * 3 + 1] * B[c * 3 + 1] + A[r * 3 + 2] * B[c * 3 + 2];
#pragma unroll
    for (int i = 0; i < 9; ++i) C[i] = t[i];
}

template <typename R>
MPM_HD R dot9(const R* A, const R* B)
{
    R s = 0;
#pragma unroll
    for (int i = 0; i < 9; ++i) s += A[i] * B[i];
    return s;
}

// det(F) - 1 through D = F - I (no cancellation for F near I)
template <typename R>
MPM_HD R det_minus_one(const R* F)
{
    R d0 = F[0] - R(1), d4 = F[4] - R(1), d8 = F[8] - R(1);
    R tr = d0 + d4 + d8;
    R m2 = (d0 * d4 - F[1] * F[3]) + (d0 * d8 - F[2] * F[6]) + (d4 * d8 - F[5] * F[7]);
    R D[9] = {d0, F[1], F[2], F[3], d4, F[5], F[6], F[7], d8};
    return tr + m2 + det3(D);
}

// ------------------------------------------------------------- B-splines

// cubic B-spline N(x) and N'(x), DiffMPMLib3D/Interpolation.h:5-30
template <typename R>
MPM_HD R cubic_w(R x, R& slope)
{
    R ax = fabs(x);
    if (ax < R(1)) {
        slope = R(1.5) * x * ax - R(2) * x;
        return R(0.5) * ax * ax * ax - ax * ax + R(2) / R(3);
    }
    if (ax < R(2)) {
        R t = R(2) - ax;
        slope = -x * ax / R(2) + R(2) * x - R(2) * x / ax;
        return t * t * t / R(6);
    }
    slope = R(0);
    return R(0);
}

// quadratic B-spline (optional kernel)
template <typename R>
MPM_HD R quad_w(R x, R& slope)
{
    R ax = fabs(x);
    if (ax < R(0.5)) {
        slope = R(-2) * x;
        return R(0.75) - x * x;
    }
    if (ax < R(1.5)) {
        R t = R(1.5) - ax;
        slope = x > R(0) ? -t : t;
        return R(0.5) * t * t;
    }
    slope = R(0);
    return R(0);
}

// Per-particle stencil: base node index and per-axis weights, slopes and
// offsets dg = x_node - x_p (node position min + i*dx as in Grid.cpp:7-26).
template <typename R, int K>
struct Stencil {
    int base[3];
    R w[3][K];
    R s[3][K];
    R g[3][K];
};

// FP32 stencil from the fractional cell coordinate f: each stencil offset
// always falls on the same piece of the spline, so weights and slopes are
// fixed polynomials in f (no divides, no branches), and dg = (o - 1 - f) dx
// (cubic) or (o - f) dx (quadratic).  Same values as Interpolation.h:5-30
// evaluated at dg/dx, up to FP32 rounding.
template <int K>
MPM_HD void make_stencil_poly(const float* x, const float* gmin, float dx, float inv_dx, Stencil<float, K>& st,
                              bool want_slope)
{
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float rel = (x[a] - gmin[a]) * inv_dx;
        if (K == 4) {
            const float fl = floorf(rel);
            const float f = rel - fl, g = 1.f - f;
            const float f2 = f * f, g2 = g * g;
            st.base[a] = (int)fl - 1;
            st.w[a][0] = g2 * g * (1.f / 6.f);
            st.w[a][1] = (0.5f * f - 1.f) * f2 + (2.f / 3.f);
            st.w[a][2] = (0.5f * g - 1.f) * g2 + (2.f / 3.f);
            st.w[a][K - 1] = f2 * f * (1.f / 6.f);
            st.g[a][0] = (-1.f - f) * dx;
            st.g[a][1] = -f * dx;
            st.g[a][2] = g * dx;
            st.g[a][K - 1] = (2.f - f) * dx;
            if (want_slope) {
                st.s[a][0] = 0.5f * g2;
                st.s[a][1] = (2.f - 1.5f * f) * f;
                st.s[a][2] = (1.5f * g - 2.f) * g;
                st.s[a][K - 1] = -0.5f * f2;
            }
        } else {
            const float fl = floorf(rel - 0.5f);
            const float f = rel - fl;  // in [0.5, 1.5)
            const float u = 1.5f - f, v = f - 1.f, z = f - 0.5f;
            st.base[a] = (int)fl;
            st.w[a][0] = 0.5f * u * u;
            st.w[a][1] = 0.75f - v * v;
            st.w[a][2] = 0.5f * z * z;
            st.g[a][0] = -f * dx;
            st.g[a][1] = (1.f - f) * dx;
            st.g[a][2] = (2.f - f) * dx;
            if (want_slope) {
                st.s[a][0] = u;
                st.s[a][1] = 2.f * v;
                st.s[a][2] = -z;
            }
        }
        if (!want_slope)
#pragma unroll
            for (int o = 0; o < K; ++o) st.s[a][o] = 0.f;
    }
}

template <typename R, int K>
MPM_HD void make_stencil_ref(const R* x, const R* gmin, R dx, R inv_dx, Stencil<R, K>& st, bool want_slope);

// Stencil of particle x: the FP32 path uses the polynomial form above, the
// FP64 path the reference's own sequence (node position, dg, N(dg/dx)).
template <typename R, int K>
MPM_HD void make_stencil(const R* x, const R* gmin, R dx, R inv_dx, Stencil<R, K>& st, bool want_slope)
{
    if constexpr (sizeof(R) == 4) make_stencil_poly<K>(x, gmin, dx, inv_dx, st, want_slope);
    else make_stencil_ref<R, K>(x, gmin, dx, inv_dx, st, want_slope);
}

template <typename R, int K>
MPM_HD void make_stencil_ref(const R* x, const R* gmin, R dx, R inv_dx, Stencil<R, K>& st, bool want_slope)
{
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        R rel = (x[a] - gmin[a]) / dx;
        int b = (K == 4) ? (int)floor(rel) - 1 : (int)floor(rel - R(0.5));
        st.base[a] = b;
#pragma unroll
        for (int o = 0; o < K; ++o) {
            R node = gmin[a] + R(b + o) * dx;
            R dg = node - x[a];
            R sl;
            st.g[a][o] = dg;
            st.w[a][o] = (K == 4) ? cubic_w(dg / dx, sl) : quad_w(dg / dx, sl);
            st.s[a][o] = want_slope ? sl : R(0);
        }
    }
}

// Reciprocal: correctly rounded in both precisions, but for FP32 without
// the full IEEE division sequence.
MPM_HD float rcp(float x)
{
#ifdef __CUDA_ARCH__
    return __frcp_rn(x);
#else
    return 1.f / x;
#endif
}
MPM_HD double rcp(double x) { return 1.0 / x; }

// x^(1/4) and x^(-1/4) for the Newton scaling factor, which only needs to be
// approximate (it accelerates convergence; it does not change the limit).
MPM_HD void quarter_pow(float x, float& g, float& ig)
{
#ifdef __CUDA_ARCH__
    const float r = rsqrtf(x);  // x^-1/2
    ig = sqrtf(r);              // x^-1/4
    g = __frcp_rn(ig);
#else
    g = sqrtf(sqrtf(x));
    ig = 1.f / g;
#endif
}
MPM_HD void quarter_pow(double x, double& g, double& ig)
{
    g = sqrt(sqrt(x));
    ig = 1.0 / g;
}

// ------------------------------------------------------------ polar / SVD

// cyclic Jacobi eigen-decomposition of a symmetric matrix (double)
MPM_HD void sym_eig3(const double* Ain, double* w, double* V)
{
    double A[9];
    for (int i = 0; i < 9; ++i) {
        A[i] = Ain[i];
        V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    }
    for (int sweep = 0; sweep < 32; ++sweep) {
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
    w[0] = A[0];
    w[1] = A[4];
    w[2] = A[8];
}

// Rotation-variant polar factor through an SVD (double): R = U V^T, det R = +1,
// the sign of det F carried by the smallest singular value.  Out of line: it
// runs only for F near inversion (the FP64 guard), and keeping its code out
// of the step kernels lets the P2G transpose run 2% faster.
static __host__ __device__ __noinline__ void polar_svd(const double* F, double* Rm)
{
    double FtF[9], w[3], V[9];
    mulTN3(F, F, FtF);
    sym_eig3(FtF, w, V);
    int o0 = 0, o1 = 1, o2 = 2, t;
    if (w[o1] > w[o0]) { t = o0; o0 = o1; o1 = t; }
    if (w[o2] > w[o0]) { t = o0; o0 = o2; o2 = t; }
    if (w[o2] > w[o1]) { t = o1; o1 = o2; o2 = t; }
    int ord[3] = {o0, o1, o2};
    double Vs[9];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) Vs[r * 3 + c] = V[r * 3 + ord[c]];
    if (det3(Vs) < 0)
        for (int r = 0; r < 3; ++r) Vs[r * 3 + 2] = -Vs[r * 3 + 2];
    double u[3][3];
    for (int c = 0; c < 2; ++c)
        for (int r = 0; r < 3; ++r) u[c][r] = F[r * 3] * Vs[c] + F[r * 3 + 1] * Vs[3 + c] + F[r * 3 + 2] * Vs[6 + c];
    double n1 = sqrt(u[0][0] * u[0][0] + u[0][1] * u[0][1] + u[0][2] * u[0][2]);
    if (n1 > 1e-300) {
        for (int r = 0; r < 3; ++r) u[0][r] /= n1;
    } else {
        u[0][0] = 1; u[0][1] = 0; u[0][2] = 0;
    }
    double d = u[0][0] * u[1][0] + u[0][1] * u[1][1] + u[0][2] * u[1][2];
    for (int r = 0; r < 3; ++r) u[1][r] -= d * u[0][r];
    double n2 = sqrt(u[1][0] * u[1][0] + u[1][1] * u[1][1] + u[1][2] * u[1][2]);
    if (n2 > 1e-14 * (n1 > 1e-300 ? n1 : 1.0)) {
        for (int r = 0; r < 3; ++r) u[1][r] /= n2;
    } else {
        int k = (fabs(u[0][0]) < fabs(u[0][1])) ? (fabs(u[0][0]) < fabs(u[0][2]) ? 0 : 2)
                                                 : (fabs(u[0][1]) < fabs(u[0][2]) ? 1 : 2);
        double e[3] = {0, 0, 0};
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
        for (int c = 0; c < 3; ++c) Rm[r * 3 + c] = u[0][r] * Vs[c * 3] + u[1][r] * Vs[c * 3 + 1] + u[2][r] * Vs[c * 3 + 2];
}

// Newton stopping rule: the iteration stops once the relative step is below
// `step` (squared here).  Convergence is quadratic: the step estimates the
// previous iterate's error e, and the new iterate's error is ~e^2 / 2.  FP32:
// a relative step of 1e-4 leaves an error of ~5e-9, below FP32 rounding, so
// FP32 stops there (against 2.5e5 random F up to 60% stretch, the factor
// differs from the FP64 SVD's by at most 1.7e-7 either way, the rounding of
// F itself).  FP64 takes one more step after its 1e-8 rule.
#ifndef MPM_POLAR_STEP2_F32
#define MPM_POLAR_STEP2_F32 1e-8f
#endif
// 1: the FP32 iteration also takes the one more step (0.5-1% slower steps)
#ifndef MPM_POLAR_EXTRA_F32
#define MPM_POLAR_EXTRA_F32 0
#endif
template <typename R>
struct Tol;
template <>
struct Tol<float> {
    static constexpr float step2 = MPM_POLAR_STEP2_F32;
    static constexpr int iters = 10;
    static constexpr bool extra = MPM_POLAR_EXTRA_F32 != 0;
};
template <>
struct Tol<double> {
    static constexpr double step2 = 1e-16;
    static constexpr int iters = 30;
    static constexpr bool extra = true;
};

// Scaled Newton iteration for the polar factor (Higham 1986):
// X <- (g X + X^{-T} / g) / 2, g = sqrt(|X^{-1}|_F / |X|_F) while far away.
// Returns false when the iterate becomes singular or does not converge.
template <typename R>
MPM_HD bool polar_newton(const R* F, R* Rm)
{
    R X[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) X[i] = F[i];
    bool scale = true, last = false;
    for (int it = 0; it < Tol<R>::iters; ++it) {
        R c[9];
        cof3(X, c);
        R d = X[0] * c[0] + X[1] * c[1] + X[2] * c[2];
        if (!(d > R(0))) return false;
        R inv_d = rcp(d);
        R g = R(1), ig = R(1);
        if (scale) {
            R nx = dot9(X, X), nc = dot9(c, c) * inv_d * inv_d;
            quarter_pow(nc * rcp(nx), g, ig);
        }
        R diff = 0, ny = 0;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            R y = R(0.5) * (g * X[i] + c[i] * inv_d * ig);
            R e = y - X[i];
            diff += e * e;
            ny += y * y;
            X[i] = y;
        }
        if (diff < R(1e-4)) scale = false;
        if (last) break;
        if (diff <= Tol<R>::step2 * ny) {
            if (!Tol<R>::extra) break;
            last = true;
        }
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) Rm[i] = X[i];
    return true;
}

// Newton-Schulz iteration for the polar factor of a nearly orthogonal F:
// X <- X (3I - X^T X) / 2.  On a singular value s = 1 + d it gives
// 1 - 3 d^2 / 2 - d^3 / 2, quadratic like Newton's, but with no inverse or
// reciprocal: about 40% fewer operations per iteration.  It converges for
// every s in (0, sqrt 3); it is used only when |I - F^T F|_F^2 <= kSchulzIn
// (every s within ~20% of 1) and returns false otherwise.  E = I - X^T X is
// formed before each update; |d| ~ |E| / 2, so once |E|_F^2 is below
// kSchulzOut the update leaves an error of ~3 |E|^2 / 8 < 4e-9 and is the
// last one.
#ifndef MPM_POLAR_SCHULZ
#define MPM_POLAR_SCHULZ 1
#endif
constexpr float kSchulzIn = 0.25f, kSchulzOut = 1e-8f;
MPM_HD bool polar_schulz(const float* F, float* Rm)
{
    float X[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) X[i] = F[i];
    for (int it = 0; it < 8; ++it) {
        // E = I - X^T X (symmetric)
        float E[9];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = r; c < 3; ++c) {
                const float m = X[r] * X[c] + X[3 + r] * X[3 + c] + X[6 + r] * X[6 + c];
                E[r * 3 + c] = E[c * 3 + r] = (r == c ? 1.f : 0.f) - m;
            }
        const float e2 = E[0] * E[0] + E[4] * E[4] + E[8] * E[8] +
                         2.f * (E[1] * E[1] + E[2] * E[2] + E[5] * E[5]);
        if (it == 0 && !(e2 <= kSchulzIn)) return false;
        // X <- X + X E / 2
        float Y[9];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c)
                Y[r * 3 + c] = X[r * 3 + c] + 0.5f * (X[r * 3] * E[c] + X[r * 3 + 1] * E[3 + c] + X[r * 3 + 2] * E[6 + c]);
#pragma unroll
        for (int i = 0; i < 9; ++i) X[i] = Y[i];
        if (e2 <= kSchulzOut) {
#pragma unroll
            for (int i = 0; i < 9; ++i) Rm[i] = X[i];
            return true;
        }
    }
    return false;
}
MPM_HD bool polar_schulz(const double*, double*) { return false; }  // FP64 keeps Newton

// Branch flags some device functions can report (a null flag pointer, the
// default, compiles the reporting away): which guarded or clamped form ran.
enum {
    BR_POLAR_SVD = 1,      // polar decomposition by the FP64 SVD (FP32 Newton not used)
    BR_INV_FP64 = 2,       // det F and F^{-T} formed in FP64 (J <= 0.25)
    BR_J_CLAMP = 4,        // J clamped at 1e-6 (Elasticity.cpp:52)
    BR_DR_REGULARISED = 8  // rotation-derivative solve regularised (det A < 1e-6, Elasticity.cpp:57-117)
};

// The FP64 guard of the polar decomposition: R from the FP64 SVD of F.  Out
// of line, like the guards below: these run only for F near inversion, and
// their double temporaries would otherwise count against the registers of
// every kernel that forms the stress or its VJP.
template <typename R>
static __host__ __device__ __noinline__ void polar_guard(const R* F, R* Rm)
{
    double Fd[9], Rd[9];
    for (int i = 0; i < 9; ++i) Fd[i] = (double)F[i];
    polar_svd(Fd, Rd);
    for (int i = 0; i < 9; ++i) Rm[i] = (R)Rd[i];
}

// S = sym(R^T F), the stretch of F = R S for a known rotation factor R
template <typename R>
MPM_HD void polar_stretch(const R* F, const R* Rm, R* S)
{
    R RtF[9];
    mulTN3(Rm, F, RtF);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) S[r * 3 + c] = R(0.5) * (RtF[r * 3 + c] + RtF[c * 3 + r]);
}

// F = R S.  The FP32 path uses Newton when F is safely away from inversion
// and the FP64 SVD otherwise (the FP64 guard).
template <typename R>
MPM_HD void polar(const R* F, R* Rm, R* S, unsigned* fl = nullptr)
{
    R J = det3(F);
    R n2 = dot9(F, F);
    R ref = n2 * sqrt(n2) * R(0.19245008972987526);  // (|F|_F / sqrt 3)^3
    bool ok = (J > R(0.05) * ref) && ((MPM_POLAR_SCHULZ && polar_schulz(F, Rm)) || polar_newton(F, Rm));
    if (!ok) {
        // the guard works on copies, so the caller's arrays are never
        // address-taken (they stay in registers on the common path)
        R Fg[9], Rg[9];
        for (int i = 0; i < 9; ++i) Fg[i] = F[i];
        polar_guard(Fg, Rg);
        for (int i = 0; i < 9; ++i) Rm[i] = Rg[i];
        if (fl) *fl |= BR_POLAR_SVD;
    }
    polar_stretch(F, Rm, S);
}

// --------------------------------------------------------- constitutive

enum { MAT_FCR = 0, MAT_NEOHOOKEAN = 1 };

// Invariants shared by P and its VJP.  Jraw = det F, Jc = max(Jraw, 1e-6),
// Jm1c = Jc - 1 (from F - I when Jraw is not clamped), Fit = F^{-T}.
// Below J = 0.25 (near inversion) these are formed in FP64.
template <typename R>
struct Inv {
    R Jraw, Jc, Jm1c;
    R Fit[9];
};

// Below J = 0.25: J, the clamped J and F^{-T} in FP64 (out of line)
template <typename R>
static __host__ __device__ __noinline__ void invariants_guard(const R* F, Inv<R>& v, unsigned* fl)
{
    double Fd[9], c[9];
    for (int i = 0; i < 9; ++i) Fd[i] = (double)F[i];
    cof3(Fd, c);
    double Jd = Fd[0] * c[0] + Fd[1] * c[1] + Fd[2] * c[2];
    for (int i = 0; i < 9; ++i) v.Fit[i] = (R)(c[i] / Jd);
    double Jcd = Jd > 1e-6 ? Jd : 1e-6;
    v.Jraw = (R)Jd;
    v.Jc = (R)Jcd;
    v.Jm1c = (R)(Jcd - 1.0);
    if (fl) *fl |= BR_INV_FP64 | (Jd > 1e-6 ? 0u : (unsigned)BR_J_CLAMP);
}

template <typename R>
MPM_HD void invariants(const R* F, Inv<R>& v, unsigned* fl = nullptr)
{
    R jm1 = det_minus_one(F);
    R J = R(1) + jm1;
    if (J > R(0.25)) {
        R c[9];
        cof3(F, c);
        R inv = rcp(J);
#pragma unroll
        for (int i = 0; i < 9; ++i) v.Fit[i] = c[i] * inv;
        v.Jraw = J;
        v.Jc = J;
        v.Jm1c = jm1;
    } else {
        R Fg[9];
        for (int i = 0; i < 9; ++i) Fg[i] = F[i];
        Inv<R> g;
        unsigned f = 0;
        invariants_guard(Fg, g, &f);
        v = g;
        if (fl) *fl |= f;
    }
}

// P(F): FCR (Elasticity.cpp:45-55) or Neo-Hookean.  R/S are returned for reuse.
template <typename R>
MPM_HD void pk(int material, const R* F, R lam, R mu, const Inv<R>& iv, R* P, R* Rm, R* S, unsigned* fl = nullptr)
{
    if (material == MAT_FCR) {
        polar(F, Rm, S, fl);
        R k = lam * iv.Jm1c * iv.Jc;
#pragma unroll
        for (int i = 0; i < 9; ++i) P[i] = R(2) * mu * (F[i] - Rm[i]) + k * iv.Fit[i];
    } else {
        R lj = log(iv.Jc);
#pragma unroll
        for (int i = 0; i < 9; ++i) P[i] = mu * (F[i] - iv.Fit[i]) + lam * lj * iv.Fit[i];
    }
}

// P F^T, the stress term P2G scatters.  Where the FP32 invariants apply
// (J > 0.25) it needs no F^{-T} (F^{-T} F^T = I): FCR 2 mu (F - R) F^T +
// lam (J - 1) J I, Neo-Hookean mu (F F^T - I) + lam log(J) I.  Elsewhere
// (the FP64 guard regime) it is pk's P times F^T.
template <typename R>
MPM_HD void stress_pf(int material, const R* F, R lam, R mu, R* PF, unsigned* fl = nullptr)
{
    const R jm1 = det_minus_one(F);
    const R J = R(1) + jm1;
    if (J > R(0.25)) {
        R D[9], dg;
        if (material == MAT_FCR) {
            R Rm[9], S[9];
            polar(F, Rm, S, fl);
#pragma unroll
            for (int i = 0; i < 9; ++i) D[i] = R(2) * mu * (F[i] - Rm[i]);
            dg = lam * jm1 * J;
        } else {
#pragma unroll
            for (int i = 0; i < 9; ++i) D[i] = mu * F[i];
            dg = lam * log(J) - mu;
        }
        mulNT3(D, F, PF);
        PF[0] += dg;
        PF[4] += dg;
        PF[8] += dg;
        return;
    }
    Inv<R> iv;
    invariants(F, iv, fl);
    R P[9], Rm[9], S[9];
    pk(material, F, lam, mu, iv, P, Rm, S, fl);
    mulNT3(P, F, PF);
}

// Derivative of the polar rotation applied to G: with A = tr(S) I - S,
// A w = axial(R^T G - G^T R) and dR = R [w]x, regularising A by 1e-4 on the
// diagonal when det A < 1e-6 (Elasticity.cpp:57-117).
template <typename T>
MPM_HD void rotation_vjp(const T* Rm, const T* S, const T* G, T* dR, unsigned* fl)
{
    T A[9] = {S[4] + S[8], -S[1], -S[2], -S[1], S[0] + S[8], -S[5], -S[2], -S[5], S[0] + S[4]};
    if (fabs(det3(A)) < T(1e-6)) {
        A[0] += T(1e-4);
        A[4] += T(1e-4);
        A[8] += T(1e-4);
        if (fl) *fl |= BR_DR_REGULARISED;
    }
    T rg[9];
    mulTN3(Rm, G, rg);
    const T b3[3] = {rg[7] - rg[5], rg[2] - rg[6], rg[3] - rg[1]};
    T c[9];
    cof3(A, c);
    const T idet = rcp(A[0] * c[0] + A[1] * c[1] + A[2] * c[2]);
    const T w0 = (c[0] * b3[0] + c[3] * b3[1] + c[6] * b3[2]) * idet;
    const T w1 = (c[1] * b3[0] + c[4] * b3[1] + c[7] * b3[2]) * idet;
    const T w2 = (c[2] * b3[0] + c[5] * b3[1] + c[8] * b3[2]) * idet;
    const T W[9] = {0, -w2, w1, w2, 0, -w0, -w1, w0, 0};
    mul3(Rm, W, dR);
}

// rotation_vjp in FP64 from F itself (R, S by the FP64 SVD), out of line
template <typename R>
static __host__ __device__ __noinline__ void rotation_vjp_guard(const R* F, const R* G, R* dR, unsigned* fl)
{
    double Fd[9], Rd[9], Gd[9], Sd[9], dRd[9];
    for (int i = 0; i < 9; ++i) {
        Fd[i] = (double)F[i];
        Gd[i] = (double)G[i];
    }
    polar_svd(Fd, Rd);
    polar_stretch(Fd, Rd, Sd);
    rotation_vjp(Rd, Sd, Gd, dRd, fl);
    for (int i = 0; i < 9; ++i) dR[i] = (R)dRd[i];
}

// VJP of P(F) applied to G = dL/dP; returns dL/dF.  exact == false follows
// d2_FCE_psi_dF2_mult_by_dF (Elasticity.cpp:57-117), including its use of
// the clamped J next to the unclamped one inside d(J F^{-T})/dF.
template <typename R>
MPM_HD void pk_vjp(int material, bool exact, const R* F, R lam, R mu, const Inv<R>& iv, const R* Rm, const R* S,
                   const R* G, R* out, unsigned* fl = nullptr)
{
    const R* Fit = iv.Fit;
    R fg = dot9(Fit, G);
    R t[9], sw[9];
    mulNT3(Fit, G, t);  // Fit G^T
    mul3(t, Fit, sw);   // Fit G^T Fit
    if (material == MAT_FCR) {
        if (!exact || iv.Jraw > R(1e-6)) {
            R a = lam * iv.Jc * iv.Jc * fg + lam * iv.Jm1c * iv.Jraw * fg;
            R b = lam * iv.Jm1c * iv.Jraw;
#pragma unroll
            for (int i = 0; i < 9; ++i) out[i] = R(2) * mu * G[i] + a * Fit[i] - b * sw[i];
        } else {
            R b = lam * iv.Jm1c * iv.Jc;
#pragma unroll
            for (int i = 0; i < 9; ++i) out[i] = R(2) * mu * G[i] - b * sw[i];
        }
        // -2 mu dR: (tr S I - S) w = axial(R^T G - G^T R), dR = R [w]x
        const R A[9] = {S[4] + S[8], -S[1], -S[2], -S[1], S[0] + S[8], -S[5], -S[2], -S[5], S[0] + S[4]};
        R dR[9];
        if (sizeof(R) == 4 && fabs(det3(A)) < R(1e-6)) {
            // FP64 guard: A near singular (two signed singular values of F
            // nearly cancel, which only an inverted or near-singular F
            // reaches) makes the solve ill-conditioned, beyond what FP32
            // holds -- redo R, S and the regularised solve in FP64 from F
            R Fg[9], Gg[9], dRg[9];
            for (int i = 0; i < 9; ++i) {
                Fg[i] = F[i];
                Gg[i] = G[i];
            }
            unsigned f = 0;
            rotation_vjp_guard(Fg, Gg, dRg, &f);
            for (int i = 0; i < 9; ++i) dR[i] = dRg[i];
            if (fl) *fl |= f;
        } else {
            rotation_vjp(Rm, S, G, dR, fl);
        }
#pragma unroll
        for (int i = 0; i < 9; ++i) out[i] -= R(2) * mu * dR[i];
    } else {
        R lj = log(iv.Jc);
        R kk = (iv.Jraw > R(1e-6)) ? lam * fg : R(0);
#pragma unroll
        for (int i = 0; i < 9; ++i) out[i] = mu * G[i] + (mu - lam * lj) * sw[i] + kk * Fit[i];
    }
}

}  // namespace mpm
