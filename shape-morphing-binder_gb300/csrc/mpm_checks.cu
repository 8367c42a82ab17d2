// mpm_checks.cu -- the engine's per-particle constitutive device code, run on
// caller-given matrices.
//
// P2G and its transpose evaluate the fixed-corotated stress and its
// derivative inside the scatter/gather kernels, where a matrix near
// inversion selects the FP64 guard (SVD polar decomposition, FP64 det F and
// F^{-T}), the J clamp or the regularised rotation derivative.  A rollout
// rarely reaches those branches, so mpm_constitutive() runs exactly the same
// device functions (mpm_math.cuh: invariants, pk, pk_vjp) on n matrices and
// reports which branches each one took.  Reference: PK_FixedCorotatedElasticity
// (DiffMPMLib3D/Elasticity.cpp:45-55) and d2_FCE_psi_dF2_mult_by_dF
// (Elasticity.cpp:57-117).
#include <cuda_runtime.h>

#include <vector>

#include "../../include/mpm.h"
#include "mpm_launch.h"
#include "mpm_math.cuh"

namespace {

template <typename R>
__global__ void k_constitutive(int n, int material, int exact, const double* __restrict__ F,
                               const double* __restrict__ G, const double* __restrict__ lam,
                               const double* __restrict__ mu, double* __restrict__ P, double* __restrict__ dP,
                               int* __restrict__ branches)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    R f[9], g[9];
    for (int i = 0; i < 9; ++i) {
        f[i] = (R)F[9 * p + i];
        g[i] = (R)G[9 * p + i];
    }
    const R l = (R)lam[p], m = (R)mu[p];
    unsigned fl = 0;
    mpm::Inv<R> iv;
    mpm::invariants(f, iv, &fl);
    R pk[9], Rm[9], S[9], out[9];
    mpm::pk(material, f, l, m, iv, pk, Rm, S, &fl);
    mpm::pk_vjp(material, exact != 0, f, l, m, iv, Rm, S, g, out, &fl);
    for (int i = 0; i < 9; ++i) {
        P[9 * p + i] = (double)pk[i];
        dP[9 * p + i] = (double)out[i];
    }
    branches[p] = (int)fl;
}

int fail(int code, const char* msg)
{
    mpm::set_last_error(msg);
    return code;
}

}  // namespace

extern "C" int mpm_constitutive(int n, int precision, int material, int adjoint, const double* F, const double* G,
                                const double* lam, const double* mu, double* P, double* dP, int* branches)
{
    if (n < 0 || (n > 0 && (!F || !G || !lam || !mu || !P || !dP))) {
        return fail(MPM_ERR_ARG, "mpm_constitutive: invalid argument");
    }
    if ((precision != MPM_FP32 && precision != MPM_FP64) || (material != MPM_MAT_FCR && material != MPM_MAT_NEOHOOKEAN) ||
        (adjoint != MPM_ADJ_REFERENCE && adjoint != MPM_ADJ_EXACT)) {
        return fail(MPM_ERR_ARG, "mpm_constitutive: invalid precision, material or adjoint");
    }
    if (n == 0) return MPM_OK;
    const size_t m9 = sizeof(double) * 9 * (size_t)n, m1 = sizeof(double) * (size_t)n;
    double *dF = nullptr, *dG = nullptr, *dl = nullptr, *dm = nullptr, *dPo = nullptr, *dHo = nullptr;
    int* db = nullptr;
    int rc = MPM_OK;
    if (cudaMalloc(&dF, m9) != cudaSuccess || cudaMalloc(&dG, m9) != cudaSuccess || cudaMalloc(&dl, m1) != cudaSuccess ||
        cudaMalloc(&dm, m1) != cudaSuccess || cudaMalloc(&dPo, m9) != cudaSuccess ||
        cudaMalloc(&dHo, m9) != cudaSuccess || cudaMalloc(&db, sizeof(int) * (size_t)n) != cudaSuccess) {
        rc = fail(MPM_ERR_OOM, "mpm_constitutive: device allocation failed");
    }
    if (rc == MPM_OK) {
        cudaMemcpy(dF, F, m9, cudaMemcpyHostToDevice);
        cudaMemcpy(dG, G, m9, cudaMemcpyHostToDevice);
        cudaMemcpy(dl, lam, m1, cudaMemcpyHostToDevice);
        cudaMemcpy(dm, mu, m1, cudaMemcpyHostToDevice);
        const int T = 128, B = (n + T - 1) / T;
        const int ex = adjoint == MPM_ADJ_EXACT;
        if (precision == MPM_FP32)
            k_constitutive<float><<<B, T>>>(n, material, ex, dF, dG, dl, dm, dPo, dHo, db);
        else
            k_constitutive<double><<<B, T>>>(n, material, ex, dF, dG, dl, dm, dPo, dHo, db);
        std::vector<int> hb(n);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(P, dPo, m9, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(dP, dHo, m9, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(hb.data(), db, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = fail(MPM_ERR_CUDA, "mpm_constitutive: CUDA error");
        } else if (branches) {
            for (int i = 0; i < n; ++i) branches[i] = hb[i];
        }
    }
    cudaFree(dF);
    cudaFree(dG);
    cudaFree(dl);
    cudaFree(dm);
    cudaFree(dPo);
    cudaFree(dHo);
    cudaFree(db);
    return rc;
}
