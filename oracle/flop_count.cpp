/*
 * ORACLE -- test infrastructure only.  Not part of the product.
 *
 * Algorithmic work per element for the roofline of the element kernels: the
 * oracle's dense forward-mode scalar (a restatement of TinyAD's Double<k>,
 * include/TinyAD/Scalar.hh) evaluated over one element with an op-counting
 * passive type, so every +, -, *, / of value, gradient and full k x k Hessian
 * counts as one flop -- the work of the reference algorithm.  The PSD
 * projection's work is modelled from the cyclic Jacobi method it follows
 * (per rotation: 13 flops for the angle, 6 per affected matrix entry for the
 * row and column updates, 6 per eigenvector entry; k(k-1)/2 rotations and
 * k(k-1) flops of off-diagonal norm per sweep; 3 k^3 for rebuilding
 * V D V^T; k^2 for the diagonal-dominance test).
 * Build + run: oracle/flop_count.sh
 */
#include <array>
#include <cmath>
#include <cstdio>

static long g_flops = 0;

struct Flop
{
    double v = 0.0;
    Flop() = default;
    Flop(double x) : v(x) {}
};
inline Flop operator+(Flop a, Flop b) { ++g_flops; return a.v + b.v; }
inline Flop operator-(Flop a, Flop b) { ++g_flops; return a.v - b.v; }
inline Flop operator*(Flop a, Flop b) { ++g_flops; return a.v * b.v; }
inline Flop operator/(Flop a, Flop b) { ++g_flops; return a.v / b.v; }
inline Flop operator-(Flop a) { return -a.v; }
inline Flop& operator+=(Flop& a, Flop b) { a = a + b; return a; }
inline Flop& operator-=(Flop& a, Flop b) { a = a - b; return a; }
inline Flop& operator*=(Flop& a, Flop b) { a = a * b; return a; }
inline Flop& operator/=(Flop& a, Flop b) { a = a / b; return a; }
inline bool operator<=(Flop a, double b) { return a.v <= b; }

#include "ad_scalar.hh"

using namespace oracle;

template <typename S, int R, int C> struct M { S m[R * C]; S& operator()(int i, int j) { return m[j * R + i]; } };

// one symmetric Dirichlet element (tests/NewtonTest.cc:28-44 form), d = 2 or 3
template <int d>
static long count_symdir()
{
    constexpr int k = d * (d + 1);
    using S = AD<k, Flop>;
    std::array<S, k> x;
    for (int i = 0; i < k; ++i) x[i] = S(Flop(0.1 * i + (i % 3 == 0 ? 1.0 : 0.0)), i);
    M<double, d, d> Mri;
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) Mri(i, j) = i == j ? 1.0 : 0.1;
    g_flops = 0;
    M<S, d, d> Mm;
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) Mm(i, j) = x[(j + 1) * d + i] - x[i];
    // det
    S det;
    if (d == 2) det = Mm(0, 0) * Mm(1, 1) - Mm(1, 0) * Mm(0, 1);
    else
        det = Mm(0, 0) * (Mm(1, 1) * Mm(2, 2) - Mm(2, 1) * Mm(1, 2)) - Mm(1, 0) * (Mm(0, 1) * Mm(2, 2) - Mm(2, 1) * Mm(0, 2))
            + Mm(2, 0) * (Mm(0, 1) * Mm(1, 2) - Mm(1, 1) * Mm(0, 2));
    // inverse = adjugate * (1/det): d*d cofactor products + d*d scalings
    const S id = Flop(1.0) / det;
    M<S, d, d> Mi;
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j)
        {
            S cof = (d == 2) ? Mm((1 - j), (1 - i)) : Mm((j + 1) % 3, (i + 1) % 3) * Mm((j + 2) % 3, (i + 2) % 3)
                                                    - Mm((j + 1) % 3, (i + 2) % 3) * Mm((j + 2) % 3, (i + 1) % 3);
            Mi(i, j) = cof * id;
        }
    // |M Mr^-1|^2 + |Mr M^-1|^2
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
    return g_flops;
}

static long projection_model(int k, int sweeps)
{
    const long rot = 13 + 6L * 2 * k + 6L * k;
    return (long)k * k + sweeps * ((long)k * (k - 1) / 2 * rot + (long)k * (k - 1)) + 3L * k * k * k;
}

int main()
{
    const long e6 = count_symdir<2>(), e12 = count_symdir<3>();
    const long p6 = projection_model(6, 5), p12 = projection_model(12, 6);
    std::printf("{\"symdir_tri_k6\": {\"eval\": %ld, \"projection\": %ld, \"total\": %ld},"
                " \"symdir_tet_k12\": {\"eval\": %ld, \"projection\": %ld, \"total\": %ld}}\n",
                e6, p6, e6 + p6, e12, p12, e12 + p12);
    return 0;
}
