/*
 * ORACLE -- test infrastructure only.  Not part of the product.
 *
 * Algorithmic work per element for the roofline of the element kernels,
 * counted by running the arithmetic with op-counting scalar types (+, -, *, /
 * and sqrt count one flop each):
 *  - "eval": the library's evaluation (include/tad/Scalar.cuh, the packed
 *    symmetric forward-mode scalar, on include/tad/Energies.cuh's functor)
 *    with the translation-invariant reduction of the kernels: the first
 *    vertex is a constant, the d(N-1) others carry derivatives, and the first
 *    vertex's derivatives are recovered by the additions of
 *    lift_translation_invariant (include/tad/ElementKernels.cuh).
 *  - "projection": the library's element projection (include/tad/Projection.cuh,
 *    translation-deflated d(N-1) eigenproblem) on the Hessians of seeded
 *    random valid deformations, with an FP32-like counting type so the FP32
 *    branches run, averaged (Jacobi sweeps and clamped modes vary).
 *  - "reference_dense_eval": the same energy on the oracle's dense
 *    forward-mode scalar (a restatement of TinyAD's Double<k>,
 *    include/TinyAD/Scalar.hh: full k x k Hessian, all N vertices active),
 *    for comparison only.
 * Build + run: oracle/flop_count.sh
 */
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>

static long g_flops = 0;

template <typename V>
struct Counted
{
    V v = V(0);
    Counted() = default;
    Counted(double x) : v((V)x) {}
    explicit operator double() const { return (double)v; }
};
template <typename V> inline Counted<V> operator+(Counted<V> a, Counted<V> b) { ++g_flops; return a.v + b.v; }
template <typename V> inline Counted<V> operator-(Counted<V> a, Counted<V> b) { ++g_flops; return a.v - b.v; }
template <typename V> inline Counted<V> operator*(Counted<V> a, Counted<V> b) { ++g_flops; return a.v * b.v; }
template <typename V> inline Counted<V> operator/(Counted<V> a, Counted<V> b) { ++g_flops; return a.v / b.v; }
template <typename V> inline Counted<V> operator-(Counted<V> a) { return -a.v; }
template <typename V> inline Counted<V>& operator+=(Counted<V>& a, Counted<V> b) { a = a + b; return a; }
template <typename V> inline Counted<V>& operator-=(Counted<V>& a, Counted<V> b) { a = a - b; return a; }
template <typename V> inline Counted<V>& operator*=(Counted<V>& a, Counted<V> b) { a = a * b; return a; }
template <typename V> inline Counted<V>& operator/=(Counted<V>& a, Counted<V> b) { a = a / b; return a; }
template <typename V> inline bool operator<(Counted<V> a, Counted<V> b) { return a.v < b.v; }
template <typename V> inline bool operator>(Counted<V> a, Counted<V> b) { return a.v > b.v; }
template <typename V> inline bool operator<=(Counted<V> a, Counted<V> b) { return a.v <= b.v; }
template <typename V> inline bool operator>=(Counted<V> a, Counted<V> b) { return a.v >= b.v; }
template <typename V> inline bool operator==(Counted<V> a, Counted<V> b) { return a.v == b.v; }
template <typename V> inline bool operator!=(Counted<V> a, Counted<V> b) { return a.v != b.v; }
template <typename V> inline Counted<V> sqrt(Counted<V> a) { ++g_flops; return std::sqrt(a.v); }

using Flop = Counted<double>;    // FP64 counting type
using FlopF = Counted<float>;    // FP32-like (sizeof 4: the projection's FP32 branches)
static_assert(sizeof(FlopF) == 4, "FlopF must look like float");

#include "ad_scalar.hh"
#include "tad/Energies.cuh"
#include "tad/Projection.cuh"

/* host element seeding the library's scalar as the kernels do
   (ActiveElement<d, N, S, FirstPassive = true>) */
template <int d, int N, typename S>
struct CountElement
{
    using scalar_type = S;
    using passive_type = typename S::passive_type;
    int64_t handle;
    int32_t vh[N];
    const double* x;
    tad::Vec<S, d> variables(int v) const
    {
        int slot = -1;
        for (int i = N - 1; i >= 0; --i)
            if (vh[i] == v) slot = i;
        tad::Vec<S, d> r;
        for (int i = 0; i < d; ++i) r[i] = S(passive_type(x[d * v + i]), (slot - 1) * d + i);
        return r;
    }
};

/* additions of lift_translation_invariant: slot-0 gradient d(N-1), column
   sums d*kr*(N-1), slot-0 diagonal block d*d*(N-1) */
static long lift_flops(int d, int N)
{
    const int kr = d * (N - 1);
    return (long)d * (N - 1) + (long)d * kr * (N - 1) + (long)d * d * (N - 1);
}

/* rest parameters: Mr = identity + 0.1 off-diagonal (column-major), weight 0.5 */
template <int d>
static void rest_params(double* prm)
{
    for (int j = 0; j < d; ++j)
        for (int i = 0; i < d; ++i) prm[j * d + i] = i == j ? 1.0 : 0.1;
    prm[d * d] = 0.5;
}

template <int d>
static long library_eval(const double* xv)
{
    constexpr int N = d + 1;
    int32_t vtx[N];
    for (int i = 0; i < N; ++i) vtx[i] = i;
    double prm[d * d + 1];
    rest_params<d>(prm);
    using S = tad::Scalar<d * (N - 1), Flop, true, Flop, Flop>;
    CountElement<d, N, S> el{0, {}, xv};
    for (int i = 0; i < N; ++i) el.vh[i] = i;
    g_flops = 0;
    if constexpr (d == 2) { tad::SymmetricDirichletTri E{vtx, prm}; (void)E(el); }
    else { tad::SymmetricDirichletTet E{vtx, prm}; (void)E(el); }
    return g_flops + lift_flops(d, N);
}

template <typename S, int R, int C> struct M { S m[R * C]; S& operator()(int i, int j) { return m[j * R + i]; } };

/* one symmetric Dirichlet element (tests/NewtonTest.cc:28-44 form) on the
   oracle's dense scalar, all k = d(d+1) variables active; fills the full
   k x k Hessian values */
template <int d>
static long reference_dense_eval(const double* xv, double* hess = nullptr)
{
    constexpr int k = d * (d + 1);
    using S = oracle::AD<k, Flop>;
    std::array<S, k> x;
    for (int i = 0; i < k; ++i) x[i] = S(Flop(xv[i]), i);
    M<double, d, d> Mri;
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) Mri(i, j) = i == j ? 1.0 : 0.1;
    g_flops = 0;
    M<S, d, d> Mm;
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) Mm(i, j) = x[(j + 1) * d + i] - x[i];
    S det;
    if (d == 2) det = Mm(0, 0) * Mm(1, 1) - Mm(1, 0) * Mm(0, 1);
    else
        det = Mm(0, 0) * (Mm(1, 1) * Mm(2, 2) - Mm(2, 1) * Mm(1, 2)) - Mm(1, 0) * (Mm(0, 1) * Mm(2, 2) - Mm(2, 1) * Mm(0, 2))
            + Mm(2, 0) * (Mm(0, 1) * Mm(1, 2) - Mm(1, 1) * Mm(0, 2));
    const S id = Flop(1.0) / det;
    M<S, d, d> Mi;
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j)
        {
            S cof = (d == 2) ? Mm((1 - j), (1 - i)) : Mm((j + 1) % 3, (i + 1) % 3) * Mm((j + 2) % 3, (i + 2) % 3)
                                                    - Mm((j + 1) % 3, (i + 2) % 3) * Mm((j + 2) % 3, (i + 1) % 3);
            Mi(i, j) = cof * id;
        }
    S e = S(Flop(0.0));
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j)
        {
            S a = Mm(i, 0) * Flop(Mri(0, j));
            for (int l = 1; l < d; ++l) a = a + Mm(i, l) * Flop(Mri(l, j));
            S b = Mi(0, j) * Flop(Mri(i, 0));
            for (int l = 1; l < d; ++l) b = b + Mi(l, j) * Flop(Mri(i, l));
            e = e + a * a + b * b;
        }
    e = e * Flop(0.5);
    const long n = g_flops;
    if (hess)
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) hess[i * k + j] = e.H(i, j).v;
    return n;
}

/* Average projection flops over n seeded valid elements: the rest simplex
   (unit edges along the axes) mapped by a random A with det > 0 (d = 2:
   rotation x diag(s) x rotation, s in [0.3, 3]; d = 3: diagonal in
   [0.3, 3] plus a small shear) and a random translation. */
template <int d>
static double projection_average(int n)
{
    constexpr int N = d + 1, k = d * N;
    unsigned long long state = 0x9E3779B97F4A7C15ull;
    auto uni = [&]() {   // xorshift64*, uniform in [0, 1)
        state ^= state >> 12; state ^= state << 25; state ^= state >> 27;
        return (double)((state * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
    };
    double total = 0.0;
    for (int t = 0; t < n; ++t)
    {
        double A[d * d];
        if (d == 2)
        {
            const double a1 = 6.283185307179586 * uni(), a2 = 6.283185307179586 * uni();
            const double s1 = 0.3 + 2.7 * uni(), s2 = 0.3 + 2.7 * uni();
            const double R1[4] = {std::cos(a1), -std::sin(a1), std::sin(a1), std::cos(a1)};
            const double R2[4] = {std::cos(a2), -std::sin(a2), std::sin(a2), std::cos(a2)};
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j)
                    A[i * 2 + j] = R1[i * 2 + 0] * s1 * R2[0 * 2 + j] + R1[i * 2 + 1] * s2 * R2[1 * 2 + j];
        }
        else
        {
            for (int i = 0; i < d * d; ++i) A[i] = 0.3 * (uni() - 0.5);
            for (int i = 0; i < d; ++i) A[i * d + i] = 0.3 + 2.7 * uni();
        }
        double xv[k];
        const double t0[3] = {uni(), uni(), uni()};
        for (int v = 0; v < N; ++v)
            for (int i = 0; i < d; ++i) xv[v * d + i] = t0[i] + (v == 0 ? 0.0 : A[i * d + (v - 1)]);
        double H[k * k];
        reference_dense_eval<d>(xv, H);
        FlopF hp[k * (k + 1) / 2];
        for (int i = 0; i < k; ++i)
            for (int j = i; j < k; ++j) hp[tad::packed_index(i, j, k)] = FlopF(H[i * k + j]);
        g_flops = 0;
        tad::project_element_hessian<d, N, FlopF>(hp, FlopF(1e-9));
        total += (double)g_flops;
    }
    return total / n;
}

int main()
{
    // valid elements (det > 0, so the energy runs to the end): the unit
    // simplex with its vertex i >= 1 moved by 0.1 i along each axis
    double x6[6], x12[12];
    for (int v = 0; v < 3; ++v)
        for (int i = 0; i < 2; ++i) x6[v * 2 + i] = (v >= 1 && v - 1 == i ? 1.0 : 0.0) + 0.1 * v * (i + 1);
    for (int v = 0; v < 4; ++v)
        for (int i = 0; i < 3; ++i) x12[v * 3 + i] = (v >= 1 && v - 1 == i ? 1.0 : 0.0) + 0.05 * v * (i + 1);
    const long e6 = library_eval<2>(x6), e12 = library_eval<3>(x12);
    const long r6 = reference_dense_eval<2>(x6), r12 = reference_dense_eval<3>(x12);
    const long p6 = std::lround(projection_average<2>(2000)), p12 = std::lround(projection_average<3>(500));
    std::printf("{\"symdir_tri_k6\": {\"eval\": %ld, \"projection\": %ld, \"total\": %ld, \"reference_dense_eval\": %ld},"
                " \"symdir_tet_k12\": {\"eval\": %ld, \"projection\": %ld, \"total\": %ld, \"reference_dense_eval\": %ld}}\n",
                e6, p6, e6 + p6, r6, e12, p12, e12 + p12, r12);
    return 0;
}
