// Host check of the FP32 polar factor (the device code of mpm_math.cuh,
// compiled for the host): Newton-Schulz, scaled Newton and the guarded
// polar() against the FP64 Jacobi-SVD factor, on seeded random F = Q (I + e H)
// with Q a random rotation and H a random symmetric matrix, e up to 0.6.
// Prints one line per regime and exits non-zero if an error bound fails.
#include <cmath>
#include <cstdio>
#include <random>

#include "mpm_math.cuh"

using namespace mpm;

namespace {

void random_f(std::mt19937& rng, double emax, double* F)
{
    std::normal_distribution<double> nd(0, 1);
    std::uniform_real_distribution<double> ud(0, 1);
    const double e = emax * ud(rng);
    double H[9], S[9], Q[9];
    for (double& h : H) h = nd(rng);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) S[r * 3 + c] = (r == c) + e * 0.5 * (H[r * 3 + c] + H[c * 3 + r]);
    double ax[3] = {nd(rng), nd(rng), nd(rng)};
    const double n = std::sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
    for (double& a : ax) a /= n;
    const double th = 3.141592653589793 * ud(rng), cs = std::cos(th), sn = std::sin(th);
    const double K[9] = {0, -ax[2], ax[1], ax[2], 0, -ax[0], -ax[1], ax[0], 0};
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            double k2 = 0;
            for (int k = 0; k < 3; ++k) k2 += K[r * 3 + k] * K[k * 3 + c];
            Q[r * 3 + c] = (r == c) + sn * K[r * 3 + c] + (1 - cs) * k2;
        }
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            double f = 0;
            for (int k = 0; k < 3; ++k) f += Q[r * 3 + k] * S[k * 3 + c];
            F[r * 3 + c] = f;
        }
}

double max_diff(const float* a, const double* b)
{
    double e = 0;
    for (int i = 0; i < 9; ++i) e = std::fmax(e, std::fabs((double)a[i] - b[i]));
    return e;
}

}  // namespace

int main()
{
    std::mt19937 rng(20251204);
    int fails = 0;
    for (double emax : {0.02, 0.1, 0.3, 0.6}) {
        double e_ns = 0, e_nw = 0, e_pol = 0, e_s = 0;
        int n = 0, n_ns = 0;
        for (int t = 0; t < 20000; ++t) {
            double Fd[9];
            random_f(rng, emax, Fd);
            float F[9];
            double Fr[9];
            for (int i = 0; i < 9; ++i) {
                F[i] = (float)Fd[i];
                Fr[i] = (double)F[i];
            }
            if (det3(Fr) <= 0.0) continue;
            ++n;
            double Rd[9], Sd[9];
            polar_svd(Fr, Rd);
            polar_stretch(Fr, Rd, Sd);
            float R1[9], R2[9], R3[9], S3[9];
            if (polar_schulz(F, R1)) {
                ++n_ns;
                e_ns = std::fmax(e_ns, max_diff(R1, Rd));
            }
            if (polar_newton(F, R2)) e_nw = std::fmax(e_nw, max_diff(R2, Rd));
            polar(F, R3, S3);
            e_pol = std::fmax(e_pol, max_diff(R3, Rd));
            double ns = 0;
            for (int i = 0; i < 9; ++i) ns = std::fmax(ns, std::fabs(Sd[i]));
            e_s = std::fmax(e_s, max_diff(S3, Sd) / ns);
        }
        std::printf("stretch <= %.2f: %d cases; Newton-Schulz %d, max |R - R64| %.2e; Newton %.2e; "
                    "polar() %.2e, S rel %.2e\n",
                    emax, n, n_ns, e_ns, e_nw, e_pol, e_s);
        // FP32 rounding of F alone moves R by ~1e-7
        if (!(e_ns < 5e-7 && e_nw < 5e-7 && e_pol < 5e-7 && e_s < 5e-7)) ++fails;
        if (emax <= 0.02 && n_ns != n) ++fails;  // near-identity F always takes Newton-Schulz
    }
    return fails ? 1 : 0;
}
