// Host check of the translation-deflated element projection of
// include/tad/Projection.cuh against the general k x k projection (the rule of
// TinyAD's project_positive_definite, HessianProjection.hh:16-101), compiled
// with g++ from the header the device kernels use.
//   * translation-invariant symmetric matrices H = P S P (P projects out the
//     d translations of the N vertices; S random, indefinite): the deflated
//     form must be taken and agree with the general projection, in FP64 to
//     rounding and in FP32 at FP32 accuracy, for eps > 0 and eps < 0 (flip);
//   * one vertex unused (zero rows and columns): still invariant, same result;
//   * the variant for matrices known to be invariant (no row-sum test) gives
//     the same result;
//   * general matrices (S itself): the deflated form must decline (-1) and
//     leave the matrix untouched.
// Prints one line "name max_error" per check; exits non-zero on failure.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "tad/Projection.cuh"

using namespace tad;

static int failures = 0;

static void report(const char* name, double err, double bound)
{
    std::printf("%s %.3e (bound %.1e)\n", name, err, bound);
    if (!(err <= bound)) ++failures;
}

template <int d, int N>
static void check(std::mt19937_64& rng, int trials)
{
    constexpr int k = d * N, NP = k * (k + 1) / 2;
    std::normal_distribution<double> nd(0.0, 1.0);
    double e64 = 0, e32 = 0, eflip = 0, eunused = 0;
    int declined = 0, wrongly_declined = 0, touched = 0;
    for (int t = 0; t < trials; ++t)
    {
        // S = sum_l +-10^((l - k/2)/2) m_l m_l^T: indefinite, eigenvalues spread over decades
        std::vector<double> S(k * k, 0.0), M(k * k);
        for (int i = 0; i < k * k; ++i) M[i] = nd(rng);
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j)
            {
                double s = 0;
                for (int l = 0; l < k; ++l) s += M[i * k + l] * M[j * k + l] * (l % 2 ? -1.0 : 1.0) * std::pow(10.0, (l - k / 2) * 0.5);
                S[i * k + j] = s;
            }
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < i; ++j) S[i * k + j] = S[j * k + i] = 0.5 * (S[i * k + j] + S[j * k + i]);
        // P = I - sum_p t_p t_p^T
        std::vector<double> P(k * k, 0.0);
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j)
                P[i * k + j] = (i == j ? 1.0 : 0.0) - ((i % d) == (j % d) ? 1.0 / N : 0.0);
        std::vector<double> PS(k * k, 0.0), H(k * k, 0.0);
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j)
                for (int l = 0; l < k; ++l) PS[i * k + j] += P[i * k + l] * S[l * k + j];
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j)
                for (int l = 0; l < k; ++l) H[i * k + j] += PS[i * k + l] * P[l * k + j];
        const bool unused = N > 2 && (t % 5 == 4);   // with N = 2 an unused vertex leaves H = 0
        if (unused)   // vertex N-1 unused: zero rows and columns, the rest invariant over N-1 vertices
        {
            std::vector<double> Pu(k * k, 0.0);
            for (int i = 0; i < k; ++i)
                for (int j = 0; j < k; ++j)
                {
                    const bool in = i / d < N - 1 && j / d < N - 1;
                    Pu[i * k + j] = in ? ((i == j ? 1.0 : 0.0) - ((i % d) == (j % d) ? 1.0 / (N - 1) : 0.0)) : 0.0;
                }
            std::fill(PS.begin(), PS.end(), 0.0);
            std::fill(H.begin(), H.end(), 0.0);
            for (int i = 0; i < k; ++i)
                for (int j = 0; j < k; ++j)
                    for (int l = 0; l < k; ++l) PS[i * k + j] += Pu[i * k + l] * S[l * k + j];
            for (int i = 0; i < k; ++i)
                for (int j = 0; j < k; ++j)
                    for (int l = 0; l < k; ++l) H[i * k + j] += PS[i * k + l] * Pu[l * k + j];
        }
        double hp[NP], ref[NP], hmax = 0;
        for (int i = 0; i < k; ++i)
            for (int j = i; j < k; ++j) { hp[packed_index(i, j, k)] = H[i * k + j]; hmax = std::fmax(hmax, std::fabs(H[i * k + j])); }
        for (double eps : {1e-9, -1.0})
        {
            for (int q = 0; q < NP; ++q) ref[q] = hp[q];
            project_positive_definite<k, double>(ref, eps);
            double a[NP];
            for (int q = 0; q < NP; ++q) a[q] = hp[q];
            const int r = project_translation_deflated<d, N, double>(a, eps);
            if (r < 0) { ++wrongly_declined; continue; }
            double err = 0;
            for (int q = 0; q < NP; ++q) err = std::fmax(err, std::fabs(a[q] - ref[q]));
            // the variant for matrices known invariant by construction (no row-sum test)
            double kn[NP];
            for (int q = 0; q < NP; ++q) kn[q] = hp[q];
            if (project_translation_deflated<d, N, double, true>(kn, eps) < 0) ++wrongly_declined;
            for (int q = 0; q < NP; ++q) err = std::fmax(err, std::fabs(kn[q] - ref[q]));
            if (eps > 0) { if (unused) eunused = std::fmax(eunused, err / hmax); else e64 = std::fmax(e64, err / hmax); }
            else eflip = std::fmax(eflip, err / hmax);
            if (eps > 0)
            {
                float f[NP];
                for (int q = 0; q < NP; ++q) f[q] = (float)hp[q];
                if (project_translation_deflated<d, N, float>(f, (float)eps) < 0) { ++wrongly_declined; continue; }
                double ef = 0;
                for (int q = 0; q < NP; ++q) ef = std::fmax(ef, std::fabs((double)f[q] - ref[q]));
                e32 = std::fmax(e32, ef / hmax);
            }
        }
        // the general matrix S itself: not invariant, must be declined untouched
        double g[NP], g0[NP];
        for (int i = 0; i < k; ++i)
            for (int j = i; j < k; ++j) g[packed_index(i, j, k)] = g0[packed_index(i, j, k)] = S[i * k + j];
        if (project_translation_deflated<d, N, double>(g, 1e-9) < 0) ++declined;
        for (int q = 0; q < NP; ++q) touched += g[q] != g0[q];
    }
    char name[96];
    std::snprintf(name, sizeof name, "d%d_N%d_fp64_vs_general", d, N); report(name, e64, 1e-13);
    std::snprintf(name, sizeof name, "d%d_N%d_fp64_flip_vs_general", d, N); report(name, eflip, 1e-13);
    std::snprintf(name, sizeof name, "d%d_N%d_unused_vertex", d, N); report(name, eunused, 1e-13);
    std::snprintf(name, sizeof name, "d%d_N%d_fp32_vs_general", d, N); report(name, e32, 1e-5);
    std::snprintf(name, sizeof name, "d%d_N%d_invariant_declined", d, N); report(name, wrongly_declined, 0);
    std::snprintf(name, sizeof name, "d%d_N%d_general_accepted", d, N); report(name, trials - declined, 0);
    std::snprintf(name, sizeof name, "d%d_N%d_general_touched", d, N); report(name, touched, 0);
}

int main()
{
    std::mt19937_64 rng(17);
    check<1, 2>(rng, 400);
    check<1, 3>(rng, 400);
    check<2, 2>(rng, 400);
    check<2, 3>(rng, 400);
    check<3, 3>(rng, 300);
    check<3, 4>(rng, 200);
    check<2, 5>(rng, 100);
    return failures ? 1 : 0;
}
