// Host check of the lane-split evaluation of elements with 9 reduced
// derivatives (the tetrahedron), compiled with g++ from the headers the
// device kernels use (include/tad/Element.cuh, Energies.cuh, Scalar.cuh):
//   * the 12 index triples of plane_line cover every pair of the 9 reduced
//     indices exactly once, and the 3 triples of direction 0 partition them;
//   * on random valid tetrahedra, the 12 Scalar<3> evaluations seeded by
//     SubsetElement give the reduced Hessian, gradient and value of one dense
//     Scalar<9> evaluation of the same functor (FP64: to rounding), also with
//     the positions staged relative to the first vertex;
//   * the FP32 lanes with staged positions (what k_elem_hess_lanes runs)
//     agree with the FP64 Hessian at FP32 accuracy.
// Prints one line "name max_error" per check; exits non-zero on failure.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>

#include "tad/Element.cuh"
#include "tad/Energies.cuh"

using namespace tad;

static int failures = 0;

static void report(const char* name, double err, double bound)
{
    std::printf("%s %.3e (bound %.1e)\n", name, err, bound);
    if (!(err <= bound)) ++failures;
}

/* the dense reduced evaluation: slot 0 constant, slots 1..3 carry derivatives
   (s - 1) * 3 + i, as ActiveElement<3, 4, S, true> seeds them */
template <typename S>
struct DenseElement
{
    using scalar_type = S;
    using passive_type = typename S::passive_type;
    static constexpr bool active_mode = true;
    int64_t handle = 0;
    int32_t vh[4] = {0, 1, 2, 3};
    const double* x = nullptr;
    Vec<S, 3> variables(int v) const
    {
        int slot = 0;
        for (int i = 3; i >= 0; --i)
            if (vh[i] == v) slot = i;
        Vec<S, 3> r;
        for (int i = 0; i < 3; ++i) r[i] = S((passive_type)x[3 * v + i], (slot - 1) * 3 + i);
        return r;
    }
};

int main()
{
    // 1. the lines
    {
        int pair_count[9][9] = {};
        int diag_dir0[9] = {};
        for (int l = 0; l < 12; ++l)
        {
            int t[3];
            plane_line(l, t);
            for (int p = 0; p < 3; ++p)
            {
                if (l < 3) ++diag_dir0[t[p]];
                for (int q = p + 1; q < 3; ++q) ++pair_count[t[p]][t[q]], ++pair_count[t[q]][t[p]];
            }
        }
        int bad = 0;
        for (int i = 0; i < 9; ++i)
        {
            bad += diag_dir0[i] != 1;
            for (int j = 0; j < 9; ++j)
                if (i != j) bad += pair_count[i][j] != 1;
        }
        report("plane_lines_cover_pairs_once", bad, 0);
    }
    // 2. lanes against the dense evaluation
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> u(-0.15, 0.15);
    const int32_t vtx[4] = {0, 1, 2, 3};
    double e64 = 0, e64s = 0, g64 = 0, f64 = 0, e32 = 0;
    for (int trial = 0; trial < 200; ++trial)
    {
        // a regular-ish tetrahedron away from the origin, jittered, and its rest shape
        double x[12] = {10, -7, 3, 11, -7, 3, 10, -6, 3, 10, -7, 4};
        double rest[12] = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1};
        for (int i = 0; i < 12; ++i) { x[i] += u(rng); rest[i] += u(rng); }
        double prm[10];
        for (int j = 0; j < 3; ++j)
            for (int i = 0; i < 3; ++i) prm[j * 3 + i] = rest[3 * (j + 1) + i] - rest[i];   // Mr, column-major
        prm[9] = 1.0 / 6.0;
        SymmetricDirichletTet E{vtx, prm};
        using D9 = Scalar<9, double, true>;
        DenseElement<D9> de;
        de.x = x;
        const D9 ref = E(de);
        if (!std::isfinite(ref.val)) continue;
        double hmax = 0, gmax = 0;
        for (int q = 0; q < 45; ++q) hmax = std::fmax(hmax, std::fabs(ref.hess[q]));
        for (int i = 0; i < 9; ++i) gmax = std::fmax(gmax, std::fabs(ref.grad[i]));
        double xs64[12];
        float xsf[12];
        for (int i = 0; i < 12; ++i)
        {
            xs64[i] = x[i] - x[i % 3];
            xsf[i] = (float)xs64[i];
        }
        for (int l = 0; l < 12; ++l)
        {
            int t[3];
            plane_line(l, t);
            using D3 = Scalar<3, double, true>;
            using F3 = Scalar<3, float, true>;
            SubsetElement<3, 4, D3, true, false> a;
            SubsetElement<3, 4, D3, true, true> b;
            SubsetElement<3, 4, F3, true, true> c;
            for (int i = 0; i < 4; ++i) a.vh[i] = b.vh[i] = c.vh[i] = vtx[i];
            for (int p = 0; p < 3; ++p) a.idx[p] = b.idx[p] = c.idx[p] = t[p];
            a.x = b.x = c.x = x;
            a.err = b.err = c.err = nullptr;
            b.xs = xs64;
            c.xs = xsf;
            const D3 ra = E(a), rb = E(b);
            const F3 rc = E(c);
            f64 = std::fmax(f64, std::fabs(ra.val - ref.val) / std::fabs(ref.val));
            for (int p = 0; p < 3; ++p)
            {
                g64 = std::fmax(g64, std::fabs(ra.grad[p] - ref.grad[t[p]]) / gmax);
                for (int q = p; q < 3; ++q)
                {
                    const double h = ref.H(t[p], t[q]);
                    e64 = std::fmax(e64, std::fabs(ra.H(p, q) - h) / hmax);
                    e64s = std::fmax(e64s, std::fabs(rb.H(p, q) - h) / hmax);
                    e32 = std::fmax(e32, std::fabs((double)rc.H(p, q) - h) / hmax);
                }
            }
        }
    }
    report("lanes_fp64_hessian_vs_dense", e64, 1e-13);
    report("lanes_fp64_gradient_vs_dense", g64, 1e-13);
    report("lanes_fp64_value_vs_dense", f64, 1e-14);
    report("lanes_fp64_staged_hessian_vs_dense", e64s, 1e-11);
    report("lanes_fp32_staged_hessian_vs_dense", e32, 2e-5);
    return failures == 0 ? 0 : 1;
}
