// Host check of the double-float arithmetic of include/tad/Scalar.cuh (the
// mixed-precision value and gradient channels) and of the mixed scalar on the
// symmetric Dirichlet triangle energy against Double<6>.  Built with g++ by
// tests/test_doublefloat_cpu.py; prints one line "name max_error" per check
// and exits non-zero if a bound is exceeded.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <limits>
#include <random>
#include <vector>

#include "tad/Energies.cuh"

using namespace tad;
using LD = long double;

static int failures = 0;

static void report(const char* name, double err, double bound)
{
    std::printf("%s %.3e (bound %.1e)\n", name, err, bound);
    if (!(err <= bound)) ++failures;
}

static LD to_ld(DoubleFloatValue a) { return (LD)a.hi + (LD)a.lo; }

static double rel(LD got, LD ref) { return (double)(std::fabs(got - ref) / std::fmax(std::fabs(ref), (LD)1e-300)); }

// host element seeding Scalar variables in first-access order, as ActiveElement does
template <int d, int N, typename S>
struct HostElement
{
    using scalar_type = S;
    using passive_type = typename S::passive_type;
    int64_t handle;
    int32_t vh[N];
    const double* x;
    Vec<S, d> variables(int v) const
    {
        int slot = -1;
        for (int i = N - 1; i >= 0; --i)
            if (vh[i] == v) slot = i;
        Vec<S, d> r;
        for (int i = 0; i < d; ++i) r[i] = S((passive_type)x[d * v + i], slot * d + i);
        return r;
    }
};

int main()
{
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> mant(-1.0, 1.0);
    std::uniform_int_distribution<int> expo(-20, 20);
    auto draw = [&]() { return std::ldexp(mant(rng), expo(rng)); };

    // 1. arithmetic: inputs are double-float splits of random doubles, the
    //    reference is long double arithmetic on the same splits
    double e_add = 0, e_mul = 0, e_div = 0, e_sqrt = 0, e_cancel = 0;
    for (int t = 0; t < 200000; ++t)
    {
        const DoubleFloatValue a(draw()), b(draw());
        const LD A = to_ld(a), B = to_ld(b);
        // addition: error relative to |a| + |b| (the bound of an accurate double-float sum)
        e_add = std::fmax(e_add, (double)(std::fabs(to_ld(a + b) - (A + B)) / (std::fabs(A) + std::fabs(B))));
        e_mul = std::fmax(e_mul, rel(to_ld(a * b), A * B));
        e_div = std::fmax(e_div, rel(to_ld(a / b), A / B));
        const DoubleFloatValue pa = fabs(a);
        e_sqrt = std::fmax(e_sqrt, rel(to_ld(sqrt(pa)), std::sqrt(to_ld(pa))));
        // a determinant-like difference with cancellation: (a b) - (a b (1 + 2^-30))
        // (the reference is formed part-wise: hi + lo of a product can span more
        // bits than an x86 long double holds, hi - hi and lo - lo cannot)
        const DoubleFloatValue c = a * b, cc = c * DoubleFloatValue(1.0 + std::ldexp(1.0, -30));
        const LD diff = ((LD)c.hi - (LD)cc.hi) + ((LD)c.lo - (LD)cc.lo);
        e_cancel = std::fmax(e_cancel, rel(to_ld(c - cc), diff));
    }
    report("dfv_add_rel_to_operands", e_add, 1e-13);
    report("dfv_mul_rel", e_mul, 1e-13);
    report("dfv_div_rel", e_div, 1e-13);
    report("dfv_sqrt_rel", e_sqrt, 1e-13);
    report("dfv_cancellation_rel", e_cancel, 1e-13);

    // 2. non-finite propagation (IEEE semantics of the double value channel)
    const DoubleFloatValue inf(std::numeric_limits<double>::infinity()), one(1.0), zero(0.0);
    int bad = 0;
    bad += !((double)(inf + one) == INFINITY);
    bad += !((double)(one - inf) == -INFINITY);
    bad += !((double)(inf * DoubleFloatValue(2.0)) == INFINITY);
    bad += !((double)(one / zero) == INFINITY);
    bad += !((double)(one / inf) == 0.0);
    bad += !std::isnan((double)(inf - inf));
    bad += !std::isnan((double)(zero / zero));
    bad += !std::isnan((double)sqrt(DoubleFloatValue(-1.0)));
    bad += !((double)sqrt(inf) == INFINITY);
    bad += !(DoubleFloatValue(1.0) < DoubleFloatValue(1.0 + 1e-12));
    bad += !(DoubleFloatValue(-0.0) <= DoubleFloatValue(0.0));
    report("dfv_special_values_wrong", bad, 0);

    // 3. the mixed scalar (double-float value and gradient, FP32 Hessian)
    //    against Double<6> on symmetric Dirichlet triangles with random
    //    shapes and rest frames
    const int NT = 2000;
    std::vector<int32_t> F(3 * NT);
    std::vector<double> P(5 * NT), X(6 * NT);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    for (int e = 0; e < NT; ++e)
    {
        for (int i = 0; i < 3; ++i) F[3 * e + i] = 3 * e + i;
        // rest triangle: a positively oriented perturbation of the reference triangle
        const double r0 = 1.0 + 0.3 * u(rng), r1 = 0.2 * u(rng), r2 = 0.3 * u(rng), r3 = 1.0 + 0.3 * u(rng);
        const double rdet = r0 * r3 - r1 * r2;
        P[5 * e + 0] = r0; P[5 * e + 1] = r1; P[5 * e + 2] = r2; P[5 * e + 3] = r3;
        P[5 * e + 4] = 1.0 / rdet;
        const double ox = 10.0 * u(rng), oy = 10.0 * u(rng);
        X[6 * e + 0] = ox; X[6 * e + 1] = oy;
        X[6 * e + 2] = ox + 1.0 + 0.4 * u(rng); X[6 * e + 3] = oy + 0.2 * u(rng);
        X[6 * e + 4] = ox + 0.2 * u(rng); X[6 * e + 5] = oy + 1.0 + 0.4 * u(rng);
    }
    SymmetricDirichletTri E{F.data(), P.data()};
    double ef = 0, eg = 0, eh = 0;
    for (int e = 0; e < NT; ++e)
    {
        HostElement<2, 3, Double<6>> el64{e, {F[3 * e], F[3 * e + 1], F[3 * e + 2]}, X.data()};
        HostElement<2, 3, Mixed<6>> elmx{e, {F[3 * e], F[3 * e + 1], F[3 * e + 2]}, X.data()};
        const auto r64 = E(el64);
        const auto rmx = E(elmx);
        ef = std::fmax(ef, std::fabs((double)rmx.val - r64.val) / std::fabs(r64.val));
        double gs = 0, ge = 0, hs = 0, he = 0;
        for (int i = 0; i < 6; ++i)
        {
            gs = std::fmax(gs, std::fabs(r64.grad[i]));
            ge = std::fmax(ge, std::fabs((double)rmx.grad[i] - r64.grad[i]));
        }
        for (int i = 0; i < 21; ++i)
        {
            hs = std::fmax(hs, std::fabs(r64.hess[i]));
            he = std::fmax(he, std::fabs((double)rmx.hess[i] - r64.hess[i]));
        }
        eg = std::fmax(eg, ge / gs);
        eh = std::fmax(eh, he / hs);
    }
    report("mixed_symdir_tri_value_rel", ef, 1e-12);
    report("mixed_symdir_tri_gradient_rel", eg, 1e-11);
    report("mixed_symdir_tri_hessian_rel", eh, 1e-5);
    return failures == 0 ? 0 : 1;
}
