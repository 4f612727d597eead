/*
 * ORACLE -- test infrastructure only.  Not part of the product.
 *
 * CPU restatement of TinyAD's sparse per-element derivative path, used by
 * tests/ as the parity reference and by bench.py as the CPU baseline.  It is
 * written from the reference's behaviour, file by file:
 *
 *   Element access, first-access local order    include/TinyAD/Detail/Element.hh:159-260
 *   per-term eval / gradient / derivatives      include/TinyAD/Detail/ScalarObjectiveTerm.hh:162-278
 *   OpenMP parallel_for (static, max-1 threads) include/TinyAD/Detail/Parallel.hh:20-69
 *   ScalarFunction eval* + setFromTriplets      include/TinyAD/Detail/ScalarFunctionImpl.hh:256-416
 *   project_positive_definite                   include/TinyAD/Utils/HessianProjection.hh:16-101
 *   newton_direction (sparse LDL^T)             include/TinyAD/Utils/NewtonDirection.hh:25-48
 *   line_search / armijo_condition              include/TinyAD/Utils/LineSearch.hh:14-65
 *   Projected-Newton loop                       tests/NewtonTest.cc:69-75
 *
 * Third-party arithmetic the reference delegates to Eigen 3 (version
 * unpinned: apt libeigen3-dev / Homebrew / vcpkg / 3.3.9 in the reference's
 * CI) is restated from published methods, not from Eigen's code:
 *   SelfAdjointEigenSolver -> cyclic Jacobi eigenvalue iteration
 *                             (Golub & Van Loan, Matrix Computations, 8.5);
 *   SimplicialLDLT         -> up-looking sparse LDL^T (T. A. Davis, "Algorithm
 *                             849: a concise sparse Cholesky factorization
 *                             package", ACM TOMS 31(4), 2005) on a nested-
 *                             dissection ordering from BFS level structures
 *                             (A. George, "Nested dissection of a regular
 *                             finite element mesh", SIAM J. Numer. Anal. 1973);
 *   2x2 / 3x3 determinant and inverse -> adjugate / determinant.
 * The reference itself cannot be compiled here (it requires Eigen 3, which is
 * absent, and gtest from the network).
 *
 * Build: oracle/build.sh (g++ -O2 -fopenmp -ffp-contract=off), output in
 * oracle/_build/.
 */
#include "ad_scalar.hh"
#include "../include/tad.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>
#include <functional>
#include <type_traits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

static thread_local std::string g_err;

// ---------------------------------------------------------------------------
// small dense matrices (column-major), generic over AD or passive scalars
// ---------------------------------------------------------------------------
template <typename T, int R, int C>
struct Mat
{
    T m[R * C];
    T& operator()(int i, int j) { return m[j * R + i]; }
    const T& operator()(int i, int j) const { return m[j * R + i]; }
};

template <typename S, typename P, int R, int K, int C>
Mat<S, R, C> matmul(const Mat<S, R, K>& A, const Mat<P, K, C>& B)
{
    Mat<S, R, C> out;
    for (int j = 0; j < C; ++j)
        for (int i = 0; i < R; ++i)
        {
            S acc = A(i, 0) * B(0, j);
            for (int k = 1; k < K; ++k) acc = acc + A(i, k) * B(k, j);
            out(i, j) = acc;
        }
    return out;
}

template <typename P, typename S, int R, int K, int C>
Mat<S, R, C> matmul_pa(const Mat<P, R, K>& A, const Mat<S, K, C>& B)
{
    Mat<S, R, C> out;
    for (int j = 0; j < C; ++j)
        for (int i = 0; i < R; ++i)
        {
            S acc = A(i, 0) * B(0, j);
            for (int k = 1; k < K; ++k) acc = acc + A(i, k) * B(k, j);
            out(i, j) = acc;
        }
    return out;
}

template <typename S, int R, int C>
S squared_norm(const Mat<S, R, C>& A)
{
    S acc = A.m[0] * A.m[0];
    for (int i = 1; i < R * C; ++i) acc = acc + A.m[i] * A.m[i];
    return acc;
}

template <typename S> S det2(const Mat<S, 2, 2>& M) { return M(0, 0) * M(1, 1) - M(1, 0) * M(0, 1); }

template <typename S>
S det3(const Mat<S, 3, 3>& M)
{
    return M(0, 0) * (M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2))
         - M(1, 0) * (M(0, 1) * M(2, 2) - M(2, 1) * M(0, 2))
         + M(2, 0) * (M(0, 1) * M(1, 2) - M(1, 1) * M(0, 2));
}

// inverse = adjugate * (1 / det)
template <typename S>
Mat<S, 2, 2> inv2(const Mat<S, 2, 2>& M)
{
    const S id = 1.0 / det2(M);
    Mat<S, 2, 2> r;
    r(0, 0) = M(1, 1) * id;
    r(1, 0) = -M(1, 0) * id;
    r(0, 1) = -M(0, 1) * id;
    r(1, 1) = M(0, 0) * id;
    return r;
}

template <typename S>
Mat<S, 3, 3> inv3(const Mat<S, 3, 3>& M)
{
    Mat<S, 3, 3> c;   // cofactors c(i,j)
    c(0, 0) = M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2);
    c(0, 1) = M(2, 0) * M(1, 2) - M(1, 0) * M(2, 2);
    c(0, 2) = M(1, 0) * M(2, 1) - M(2, 0) * M(1, 1);
    c(1, 0) = M(2, 1) * M(0, 2) - M(0, 1) * M(2, 2);
    c(1, 1) = M(0, 0) * M(2, 2) - M(2, 0) * M(0, 2);
    c(1, 2) = M(2, 0) * M(0, 1) - M(0, 0) * M(2, 1);
    c(2, 0) = M(0, 1) * M(1, 2) - M(1, 1) * M(0, 2);
    c(2, 1) = M(1, 0) * M(0, 2) - M(0, 0) * M(1, 2);
    c(2, 2) = M(0, 0) * M(1, 1) - M(1, 0) * M(0, 1);
    const S det = M(0, 0) * c(0, 0) + M(1, 0) * c(1, 0) + M(2, 0) * c(2, 0);
    const S id = 1.0 / det;
    Mat<S, 3, 3> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r(i, j) = c(j, i) * id;
    return r;
}

// ---------------------------------------------------------------------------
// Element: variables(vh) with first-access deduplication (Element.hh:208-260)
// ---------------------------------------------------------------------------
template <int d, int N, typename S>
struct Element
{
    static constexpr int k = d * N;
    static constexpr bool active = !std::is_floating_point<S>::value;
    int64_t handle;
    const double* x;
    int64_t n_vars;
    int l2g[k];
    int n_local = 0;

    Element(int64_t h, const double* x_, int64_t n) : handle(h), x(x_), n_vars(n) {}

    std::array<S, d> variables(int vh)
    {
        const int64_t g0 = (int64_t)d * vh;
        if (vh < 0 || g0 + d > n_vars) throw std::runtime_error("variable handle out of range");
        int local = -1;
        for (int i = 0; i < n_local; i += d)
            if (l2g[i] == g0) { local = i; break; }
        if (local < 0)
        {
            if (n_local >= k) throw std::runtime_error("Too many variables requested via element.variables(...).");
            local = n_local;
            for (int i = 0; i < d; ++i) l2g[n_local++] = (int)(g0 + i);
        }
        std::array<S, d> v;
        for (int i = 0; i < d; ++i)
        {
            if constexpr (active) v[i] = S(x[g0 + i], local + i);
            else v[i] = x[g0 + i];
        }
        return v;
    }
};

// ---------------------------------------------------------------------------
// Built-in energies (tad.h enum).  Written like the reference test lambdas.
// ---------------------------------------------------------------------------
template <int d, typename S>
std::array<S, d> vsub(const std::array<S, d>& a, const std::array<S, d>& b)
{
    std::array<S, d> r;
    for (int i = 0; i < d; ++i) r[i] = a[i] - b[i];
    return r;
}

// tests/NewtonTest.cc:28-44 (weight w instead of 1/#F)
template <typename El>
auto energy_symdir_tri(El& el, const int* h, const double* prm)
{
    using S = std::remove_reference_t<decltype(el.variables(0)[0])>;
    Mat<double, 2, 2> Mr; Mr.m[0] = prm[0]; Mr.m[1] = prm[1]; Mr.m[2] = prm[2]; Mr.m[3] = prm[3];
    const double w = prm[4];
    auto a = el.variables(h[0]);
    auto b = el.variables(h[1]);
    auto c = el.variables(h[2]);
    auto ba = vsub<2, S>(b, a), ca = vsub<2, S>(c, a);
    Mat<S, 2, 2> M; M(0, 0) = ba[0]; M(1, 0) = ba[1]; M(0, 1) = ca[0]; M(1, 1) = ca[1];
    if (value_of(det2(M)) <= 0.0) return S(INFINITY);
    const Mat<double, 2, 2> Mri = inv2(Mr);
    return (squared_norm(matmul(M, Mri)) + squared_norm(matmul_pa(Mr, inv2(M)))) * w;
}

template <typename El>
auto energy_symdir_tet(El& el, const int* h, const double* prm)
{
    using S = std::remove_reference_t<decltype(el.variables(0)[0])>;
    Mat<double, 3, 3> Mr; for (int i = 0; i < 9; ++i) Mr.m[i] = prm[i];
    const double w = prm[9];
    auto a = el.variables(h[0]);
    auto b = el.variables(h[1]);
    auto c = el.variables(h[2]);
    auto dd = el.variables(h[3]);
    auto ba = vsub<3, S>(b, a), ca = vsub<3, S>(c, a), da = vsub<3, S>(dd, a);
    Mat<S, 3, 3> M;
    for (int i = 0; i < 3; ++i) { M(i, 0) = ba[i]; M(i, 1) = ca[i]; M(i, 2) = da[i]; }
    if (value_of(det3(M)) <= 0.0) return S(INFINITY);
    const Mat<double, 3, 3> Mri = inv3(Mr);
    return (squared_norm(matmul(M, Mri)) + squared_norm(matmul_pa(Mr, inv3(M)))) * w;
}

// tests/NewtonTest.cc:48-55 (weighted)
template <int d, typename El>
auto energy_penalty(El& el, const int* h, const double* prm)
{
    using S = std::remove_reference_t<decltype(el.variables(0)[0])>;
    auto p = el.variables(h[0]);
    S acc = (prm[0] - p[0]) * (prm[0] - p[0]);
    for (int i = 1; i < d; ++i) acc = acc + (prm[i] - p[i]) * (prm[i] - p[i]);
    return acc * prm[d];
}

template <int d, int N, typename El>
auto energy_quadratic(El& el, const int* h, const double* prm)
{
    using S = std::remove_reference_t<decltype(el.variables(0)[0])>;
    constexpr int k = d * N;
    std::array<S, k> x;
    for (int n = 0; n < N; ++n)
    {
        auto v = el.variables(h[n]);
        for (int i = 0; i < d; ++i) x[n * d + i] = v[i];
    }
    S acc(prm[k * k + k]);
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j)
            if (prm[i * k + j] != 0.0) acc = acc + prm[i * k + j] * x[i] * x[j];
    for (int i = 0; i < k; ++i)
        if (prm[k * k + i] != 0.0) acc = acc + prm[k * k + i] * x[i];
    return acc;
}

inline double sqr_any(double v) { return v * v; }
template <typename S> S sqr_any(const S& v) { return sqr(v); }

template <int d, typename El>
auto energy_dirichlet_tri(El& el, const int* h, const double* prm)
{
    using S = std::remove_reference_t<decltype(el.variables(0)[0])>;
    auto a = el.variables(h[0]);
    auto b = el.variables(h[1]);
    auto c = el.variables(h[2]);
    S acc = sqr_any(b[0] - a[0]);
    for (int i = 1; i < d; ++i) acc = acc + sqr_any(b[i] - a[i]);
    for (int i = 0; i < d; ++i) acc = acc + sqr_any(c[i] - b[i]);
    for (int i = 0; i < d; ++i) acc = acc + sqr_any(a[i] - c[i]);
    return prm[0] * acc;
}

// ---------------------------------------------------------------------------
// PSD projection (HessianProjection.hh:16-101) with a Jacobi eigensolver
// ---------------------------------------------------------------------------
template <int k>
bool positive_diagonally_dominant(const double* H, double eps)   // HessianProjection.hh:23-42
{
    for (int i = 0; i < k; ++i)
    {
        double off = 0.0;
        for (int j = 0; j < k; ++j)
            if (i != j) off += std::fabs(H[j * k + i]);
        if (H[i * k + i] < off + eps) return false;
    }
    return true;
}

// Cyclic Jacobi: A (k x k symmetric, column-major) -> eigenvalues ev, eigenvectors V (columns).
inline void jacobi_eigen(int k, const double* A_in, double* ev, double* V)
{
    std::vector<double> A(A_in, A_in + k * k);
    // symmetrise (the reference's eigensolver reads the lower triangle only)
    for (int j = 0; j < k; ++j)
        for (int i = j + 1; i < k; ++i)
            A[j * k + i] = A[i * k + j] = A[j * k + i];
    for (int i = 0; i < k * k; ++i) V[i] = 0.0;
    for (int i = 0; i < k; ++i) V[i * k + i] = 1.0;
    double fro = 0.0;
    for (double v : A) fro += v * v;
    fro = std::sqrt(fro);
    for (int sweep = 0; sweep < 60; ++sweep)
    {
        double off = 0.0;
        for (int q = 1; q < k; ++q)
            for (int p = 0; p < q; ++p) off += A[q * k + p] * A[q * k + p];
        if (std::sqrt(off) <= 1e-17 * fro || off == 0.0) break;
        for (int p = 0; p < k - 1; ++p)
            for (int q = p + 1; q < k; ++q)
            {
                const double apq = A[q * k + p];
                if (apq == 0.0) continue;
                const double app = A[p * k + p], aqq = A[q * k + q];
                const double theta = (aqq - app) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0);
                const double s = t * c;
                for (int r = 0; r < k; ++r)   // columns p, q of A
                {
                    const double arp = A[p * k + r], arq = A[q * k + r];
                    A[p * k + r] = c * arp - s * arq;
                    A[q * k + r] = s * arp + c * arq;
                }
                for (int r = 0; r < k; ++r)   // rows p, q of A
                {
                    const double apr = A[r * k + p], aqr = A[r * k + q];
                    A[r * k + p] = c * apr - s * aqr;
                    A[r * k + q] = s * apr + c * aqr;
                }
                A[q * k + p] = A[p * k + q] = 0.0;
                for (int r = 0; r < k; ++r)
                {
                    const double vrp = V[p * k + r], vrq = V[q * k + r];
                    V[p * k + r] = c * vrp - s * vrq;
                    V[q * k + r] = s * vrp + c * vrq;
                }
            }
    }
    for (int i = 0; i < k; ++i) ev[i] = A[i * k + i];
}

template <int k>
void project_positive_definite(double* H, double eps)            // HessianProjection.hh:48-101
{
    if (k == 0) return;
    if (positive_diagonally_dominant<k>(H, eps)) return;
    double ev[k], V[k * k];
    jacobi_eigen(k, H, ev, V);
    bool all_positive = true;
    for (int i = 0; i < k; ++i)
    {
        if (eps < 0)
        {
            if (ev[i] < 0) { ev[i] = -ev[i]; all_positive = false; }
        }
        else if (ev[i] < eps) { ev[i] = eps; all_positive = false; }
    }
    if (all_positive) return;
    for (int j = 0; j < k; ++j)
        for (int i = 0; i < k; ++i)
        {
            double acc = 0.0;
            for (int l = 0; l < k; ++l) acc += V[l * k + i] * ev[l] * V[l * k + j];
            H[j * k + i] = acc;
        }
}

// ---------------------------------------------------------------------------
// Problem
// ---------------------------------------------------------------------------
struct Term
{
    int energy, N;
    int64_t n_elem;
    std::vector<int> handles;
    std::vector<double> params;
    int n_params;
};

struct Triplet { int r, c; double v; };

struct Problem
{
    int d;
    int64_t n_handles, n_vars;
    int n_threads;
    std::vector<Term> terms;
    // last assembled Hessian (CSC)
    std::vector<int> outer, inner;
    std::vector<double> values;
    // cached symbolic LDL^T (pattern constant across Newton iterations,
    // like LinearSolver::sparsity_pattern_dirty, LinearSolver.hh:12-19)
    bool ldl_ready = false;
    std::vector<int> perm, iperm, parent, Lp, Lnz, Li;
    std::vector<double> Lx, D;
    std::vector<int> pattern_outer, pattern_inner;
    // timings of the last newton call (seconds)
    double t_eval = 0, t_assemble = 0, t_solve = 0, t_ls = 0;
};

static int get_n_threads(const Problem& p)                      // Parallel.hh:20-31
{
#ifdef _OPENMP
    if (p.n_threads >= 1) return p.n_threads;
    return std::max(1, omp_get_max_threads() - 1);
#else
    return 1;
#endif
}

template <typename F>
static void parallel_for(const Problem& p, int64_t n, F body)    // Parallel.hh:37-69
{
    std::string first_error;
    bool failed = false;
#pragma omp parallel for schedule(static) num_threads(get_n_threads(p))
    for (int64_t i = 0; i < n; ++i)
    {
        bool skip;
#pragma omp atomic read
        skip = failed;
        if (skip) continue;
        try { body(i); }
        catch (const std::exception& ex)
        {
#pragma omp critical
            {
                if (!failed) first_error = ex.what();
                failed = true;
            }
        }
    }
    if (failed) throw std::runtime_error(first_error);
}

// dispatch an energy for element e with element type El
template <int d, int N, typename El>
static auto call_energy(const Term& t, El& el, int64_t e)
{
    const int* h = &t.handles[e * t.N];
    const double* prm = t.params.data() + e * t.n_params;
    using S = std::remove_reference_t<decltype(el.variables(0)[0])>;
    switch (t.energy)
    {
    case TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI:
        if constexpr (d == 2 && N == 3) return energy_symdir_tri(el, h, prm);
        break;
    case TAD_ENERGY_SYMMETRIC_DIRICHLET_TET:
        if constexpr (d == 3 && N == 4) return energy_symdir_tet(el, h, prm);
        break;
    case TAD_ENERGY_POSITION_PENALTY:
        if constexpr (N == 1) return energy_penalty<d>(el, h, prm);
        break;
    case TAD_ENERGY_QUADRATIC:
        return energy_quadratic<d, N>(el, h, prm);
    case TAD_ENERGY_DIRICHLET_TRI:
        if constexpr (N == 3) return energy_dirichlet_tri<d>(el, h, prm);
        break;
    }
    throw std::runtime_error("energy not available for this (d, N)");
    return S(0.0);
}

// ScalarObjectiveTerm::eval (ScalarObjectiveTerm.hh:162-186)
template <int d, int N>
static double term_eval(const Problem& p, const Term& t, const double* x)
{
    std::vector<double> res(t.n_elem);
    parallel_for(p, t.n_elem, [&](int64_t e) {
        Element<d, N, double> el(t.handles[e * N], x, p.n_vars);
        el.handle = e;
        res[e] = call_energy<d, N>(t, el, e);
    });
    double f = 0.0;
    for (int64_t e = 0; e < t.n_elem; ++e) f += res[e];
    return f;
}

// ScalarObjectiveTerm::eval_with_gradient_add / eval_with_derivatives_add
// (ScalarObjectiveTerm.hh:188-278): parallel evaluation (+ projection), then a
// serial scatter in element order.
template <int d, int N>
static void term_eval_derivs(const Problem& p, const Term& t, const double* x,
                             bool hessian, bool project, double eps,
                             double& f, std::vector<double>& g, std::vector<Triplet>* trips)
{
    constexpr int k = d * N;
    using S = AD<k, double>;
    std::vector<S> res(t.n_elem);
    std::vector<std::array<int, k>> l2g(t.n_elem);
    std::vector<int> nloc(t.n_elem);
    parallel_for(p, t.n_elem, [&](int64_t e) {
        Element<d, N, S> el(e, x, p.n_vars);
        S r = call_energy<d, N>(t, el, e);
        if (hessian && project) project_positive_definite<k>(r.hess.data(), eps);
        for (int i = 0; i < k; ++i)
            if (!std::isfinite(r.grad[i])) throw std::runtime_error("non-finite gradient");
        if (hessian)
            for (int i = 0; i < k * k; ++i)
                if (!std::isfinite(r.hess[i])) throw std::runtime_error("non-finite Hessian");
        res[e] = r;
        for (int i = 0; i < el.n_local; ++i) l2g[e][i] = el.l2g[i];
        nloc[e] = el.n_local;
    });
    for (int64_t e = 0; e < t.n_elem; ++e)
    {
        f += res[e].val;
        for (int i = 0; i < nloc[e]; ++i) g[l2g[e][i]] += res[e].grad[i];
        if (trips)
            for (int i = 0; i < nloc[e]; ++i)
                for (int j = 0; j < nloc[e]; ++j)
                    trips->push_back({l2g[e][i], l2g[e][j], res[e].H(i, j)});
    }
}

#define ORACLE_DISPATCH(FN, ...)                                                         \
    switch (p.d * 100 + t.N)                                                             \
    {                                                                                    \
    case 101: FN<1, 1>(__VA_ARGS__); break;                                              \
    case 201: FN<2, 1>(__VA_ARGS__); break;                                              \
    case 301: FN<3, 1>(__VA_ARGS__); break;                                              \
    case 102: FN<1, 2>(__VA_ARGS__); break;                                              \
    case 202: FN<2, 2>(__VA_ARGS__); break;                                              \
    case 103: FN<1, 3>(__VA_ARGS__); break;                                              \
    case 203: FN<2, 3>(__VA_ARGS__); break;                                              \
    case 303: FN<3, 3>(__VA_ARGS__); break;                                              \
    case 304: FN<3, 4>(__VA_ARGS__); break;                                              \
    default: throw std::runtime_error("unsupported (var_dim, valence) in oracle");      \
    }

static double eval(const Problem& p, const double* x)            // ScalarFunctionImpl.hh:256-273
{
    double f = 0.0;
    for (const Term& t : p.terms)
    {
        if (f == INFINITY) return INFINITY;
        double ft = 0.0;
        switch (p.d * 100 + t.N)
        {
        case 101: ft = term_eval<1, 1>(p, t, x); break;
        case 201: ft = term_eval<2, 1>(p, t, x); break;
        case 301: ft = term_eval<3, 1>(p, t, x); break;
        case 102: ft = term_eval<1, 2>(p, t, x); break;
        case 202: ft = term_eval<2, 2>(p, t, x); break;
        case 103: ft = term_eval<1, 3>(p, t, x); break;
        case 203: ft = term_eval<2, 3>(p, t, x); break;
        case 303: ft = term_eval<3, 3>(p, t, x); break;
        case 304: ft = term_eval<3, 4>(p, t, x); break;
        default: throw std::runtime_error("unsupported (var_dim, valence) in oracle");
        }
        f += ft;
    }
    return f;
}

// setFromTriplets semantics: duplicates summed in insertion order, rows sorted
// within each column (ScalarFunctionImpl.hh:398).
static void triplets_to_csc(int64_t n, std::vector<Triplet>& trips, std::vector<int>& outer,
                            std::vector<int>& inner, std::vector<double>& values)
{
    std::vector<int64_t> idx(trips.size());
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) {
        if (trips[a].c != trips[b].c) return trips[a].c < trips[b].c;
        return trips[a].r < trips[b].r;
    });
    outer.assign(n + 1, 0);
    inner.clear(); values.clear();
    for (size_t q = 0; q < idx.size();)
    {
        const Triplet& t0 = trips[idx[q]];
        double v = t0.v;
        size_t r = q + 1;
        while (r < idx.size() && trips[idx[r]].c == t0.c && trips[idx[r]].r == t0.r) { v += trips[idx[r]].v; ++r; }
        inner.push_back(t0.r); values.push_back(v);
        outer[t0.c + 1]++;
        q = r;
    }
    for (int64_t c = 0; c < n; ++c) outer[c + 1] += outer[c];
}

static void eval_derivs(Problem& p, const double* x, bool hessian, bool project, double eps,
                        double& f, std::vector<double>& g)
{
    f = 0.0;
    g.assign(p.n_vars, 0.0);
    std::vector<Triplet> trips;
    for (const Term& t : p.terms)
        ORACLE_DISPATCH(term_eval_derivs, p, t, x, hessian, project, eps, f, g, hessian ? &trips : nullptr);
    if (hessian) triplets_to_csc(p.n_vars, trips, p.outer, p.inner, p.values);
}

// ---------------------------------------------------------------------------
// Nested dissection ordering on the vertex graph (BFS level-set separators)
// ---------------------------------------------------------------------------
static void nd_order(const std::vector<std::vector<int>>& adj, std::vector<int>& order)
{
    const int nv = (int)adj.size();
    std::vector<int> inset(nv, 0), visited(nv, 0), level(nv, 0);
    int set_counter = 0, visit_counter = 0;
    order.clear();
    order.reserve(nv);
    // BFS inside the vertex set set_id; lo = visit order, ls = level starts
    auto bfs = [&](int src, int set_id, std::vector<int>& lo, std::vector<int>& ls) {
        ++visit_counter;
        lo.clear(); ls.clear();
        lo.push_back(src); visited[src] = visit_counter; level[src] = 0;
        ls.push_back(0);
        for (size_t head = 0; head < lo.size(); ++head)
        {
            const int v = lo[head];
            if (level[v] != (int)ls.size() - 1) ls.push_back((int)head);
            for (int u : adj[v])
                if (inset[u] == set_id && visited[u] != visit_counter)
                {
                    visited[u] = visit_counter; level[u] = level[v] + 1; lo.push_back(u);
                }
        }
        ls.push_back((int)lo.size());
    };
    std::function<void(const std::vector<int>&)> rec = [&](const std::vector<int>& verts) {
        if (verts.size() <= 16) { order.insert(order.end(), verts.begin(), verts.end()); return; }
        const int sid = ++set_counter;
        for (int v : verts) inset[v] = sid;
        std::vector<int> lo, ls;
        bfs(verts[0], sid, lo, ls);
        bfs(lo.back(), sid, lo, ls);        // from a pseudo-peripheral vertex
        if (lo.size() < verts.size())
        {
            const int vis = visit_counter;
            std::vector<int> rest;
            for (int v : verts) if (visited[v] != vis) rest.push_back(v);
            const std::vector<int> comp = lo;
            rec(comp);
            rec(rest);
            return;
        }
        const int nlev = (int)ls.size() - 1;
        if (nlev < 3) { order.insert(order.end(), verts.begin(), verts.end()); return; }
        const int half = (int)verts.size() / 2;
        int m = 1;
        while (m < nlev - 2 && ls[m + 1] <= half) ++m;
        const std::vector<int> A(lo.begin(), lo.begin() + ls[m]);
        const std::vector<int> S(lo.begin() + ls[m], lo.begin() + ls[m + 1]);
        const std::vector<int> B(lo.begin() + ls[m + 1], lo.end());
        rec(A);
        rec(B);
        order.insert(order.end(), S.begin(), S.end());
    };
    std::vector<int> all(nv);
    std::iota(all.begin(), all.end(), 0);
    rec(all);
}

// ---------------------------------------------------------------------------
// Up-looking sparse LDL^T (Davis 2005) on P A P^T
// ---------------------------------------------------------------------------
static void ldl_symbolic(Problem& p)
{
    const int64_t n = p.n_vars;
    const int d = p.d;
    const int64_t nv = n / d;
    // vertex graph from the block pattern
    std::vector<std::vector<int>> adj(nv);
    for (int64_t c = 0; c < n; ++c)
        for (int q = p.outer[c]; q < p.outer[c + 1]; ++q)
        {
            const int vr = p.inner[q] / d, vc = (int)(c / d);
            if (vr != vc && (c % d) == 0 && (p.inner[q] % d) == 0) adj[vc].push_back(vr);
        }
    for (auto& a : adj) { std::sort(a.begin(), a.end()); a.erase(std::unique(a.begin(), a.end()), a.end()); }
    std::vector<int> vorder;
    nd_order(adj, vorder);
    p.perm.resize(n); p.iperm.resize(n);
    for (int64_t i = 0; i < nv; ++i)
        for (int j = 0; j < d; ++j) p.perm[i * d + j] = vorder[i] * d + j;
    for (int64_t i = 0; i < n; ++i) p.iperm[p.perm[i]] = (int)i;
    // permuted pattern (upper part by column: rows i <= k of column k)
    std::vector<std::vector<int>> colrows(n);
    for (int64_t c = 0; c < n; ++c)
        for (int q = p.outer[c]; q < p.outer[c + 1]; ++q)
        {
            const int i = p.iperm[p.inner[q]], k = p.iperm[c];
            if (i <= k) colrows[k].push_back(i);
        }
    p.parent.assign(n, -1);
    p.Lnz.assign(n, 0);
    std::vector<int> flag(n, -1);
    for (int64_t k = 0; k < n; ++k)
    {
        flag[k] = (int)k;
        for (int i0 : colrows[k])
            for (int i = i0; i < k && flag[i] != k; i = p.parent[i])
            {
                if (p.parent[i] == -1) p.parent[i] = (int)k;
                p.Lnz[i]++;
                flag[i] = (int)k;
            }
    }
    p.Lp.assign(n + 1, 0);
    for (int64_t k = 0; k < n; ++k) p.Lp[k + 1] = p.Lp[k] + p.Lnz[k];
    p.Li.assign(p.Lp[n], 0);
    p.Lx.assign(p.Lp[n], 0.0);
    p.D.assign(n, 0.0);
    p.pattern_outer = p.outer;
    p.pattern_inner = p.inner;
    p.ldl_ready = true;
}

static void ldl_numeric(Problem& p, double w_identity)
{
    const int64_t n = p.n_vars;
    std::vector<double> Y(n, 0.0);
    std::vector<int> flag(n, -1), pattern(n);
    std::fill(p.Lnz.begin(), p.Lnz.end(), 0);
    // permuted matrix by column (rows i <= k)
    std::vector<std::vector<std::pair<int, double>>> col(n);
    for (int64_t c = 0; c < n; ++c)
        for (int q = p.outer[c]; q < p.outer[c + 1]; ++q)
        {
            const int i = p.iperm[p.inner[q]], k = p.iperm[c];
            if (i <= k) col[k].push_back({i, p.values[q] + (i == k && p.inner[q] == c ? w_identity : 0.0)});
        }
    for (int64_t k = 0; k < n; ++k)
    {
        Y[k] = 0.0;
        int top = (int)n;
        flag[k] = (int)k;
        for (auto& iv : col[k])
        {
            int i = iv.first;
            Y[i] += iv.second;
            int len = 0;
            for (; flag[i] != k; i = p.parent[i]) { pattern[len++] = i; flag[i] = (int)k; }
            while (len > 0) pattern[--top] = pattern[--len];
        }
        double dk = Y[k];
        Y[k] = 0.0;
        for (; top < n; ++top)
        {
            const int i = pattern[top];
            const double yi = Y[i];
            Y[i] = 0.0;
            const int p2 = p.Lp[i] + p.Lnz[i];
            for (int q = p.Lp[i]; q < p2; ++q) Y[p.Li[q]] -= p.Lx[q] * yi;
            const double lki = yi / p.D[i];
            dk -= lki * yi;
            p.Li[p2] = (int)k;
            p.Lx[p2] = lki;
            p.Lnz[i]++;
        }
        if (dk == 0.0 || !std::isfinite(dk)) throw std::runtime_error("Linear solve failed.");
        p.D[k] = dk;
    }
}

static void ldl_solve(const Problem& p, const double* b, double* x)
{
    const int64_t n = p.n_vars;
    std::vector<double> y(n);
    for (int64_t i = 0; i < n; ++i) y[p.iperm[i]] = b[i];
    for (int64_t j = 0; j < n; ++j)
        for (int q = p.Lp[j]; q < p.Lp[j] + p.Lnz[j]; ++q) y[p.Li[q]] -= p.Lx[q] * y[j];
    for (int64_t j = 0; j < n; ++j) y[j] /= p.D[j];
    for (int64_t j = n - 1; j >= 0; --j)
        for (int q = p.Lp[j]; q < p.Lp[j] + p.Lnz[j]; ++q) y[j] -= p.Lx[q] * y[p.Li[q]];
    for (int64_t i = 0; i < n; ++i) x[i] = y[p.iperm[i]];
}

// newton_direction (NewtonDirection.hh:25-48): d = -(H + wI)^-1 g
static void newton_direction(Problem& p, const std::vector<double>& g, double w, std::vector<double>& d)
{
    if (p.outer.size() != (size_t)p.n_vars + 1) throw std::runtime_error("no assembled Hessian: call eval_with_hessian_proj first");
    if (!p.ldl_ready || p.pattern_outer != p.outer || p.pattern_inner != p.inner) ldl_symbolic(p);
    ldl_numeric(p, w);
    std::vector<double> mg(g.size());
    for (size_t i = 0; i < g.size(); ++i) mg[i] = -g[i];
    d.resize(g.size());
    ldl_solve(p, mg.data(), d.data());
    for (double v : d)
        if (!std::isfinite(v)) throw std::runtime_error("non-finite Newton direction");
}

// line_search (LineSearch.hh:26-65)
static bool line_search(const Problem& p, const std::vector<double>& x0, const std::vector<double>& d,
                        double f, const std::vector<double>& g, std::vector<double>& x_out, double& f_out,
                        double s_max = 1.0, double shrink = 0.8, int max_iters = 64, double armijo = 1e-4,
                        int* trials = nullptr)
{
    if (s_max <= 0.0) throw std::runtime_error("Max step size not positive.");
    const bool try_one = s_max > 1.0;
    double dg = 0.0;
    for (size_t i = 0; i < d.size(); ++i) dg += d[i] * g[i];
    std::vector<double> x_new(x0.size());
    double s = s_max;
    for (int it = 0; it < max_iters; ++it)
    {
        for (size_t i = 0; i < x0.size(); ++i) x_new[i] = x0[i] + s * d[i];
        const double f_new = eval(p, x_new.data());
        if (trials) *trials = it + 1;
        if (f_new <= f + armijo * s * dg)
        {
            x_out = x_new; f_out = f_new;
            return true;
        }
        if (try_one && s > 1.0 && s * shrink < 1.0) s = 1.0;
        else s *= shrink;
    }
    x_out = x0; f_out = f;
    return false;
}

} // namespace oracle

// ---------------------------------------------------------------------------
// C ABI of the oracle (used through ctypes by tests/ and bench.py)
// ---------------------------------------------------------------------------
using namespace oracle;

#define ORACLE_TRY(...) try { __VA_ARGS__ } catch (const std::exception& ex) { g_err = ex.what(); return 1; }

extern "C" {

__attribute__((visibility("default"))) const char* oracle_last_error() { return g_err.c_str(); }

__attribute__((visibility("default"))) void* oracle_problem_create(int d, int64_t n_handles, int n_threads)
{
    Problem* p = new Problem();
    p->d = d; p->n_handles = n_handles; p->n_vars = d * n_handles; p->n_threads = n_threads;
    return p;
}

__attribute__((visibility("default"))) void oracle_problem_destroy(void* p) { delete (Problem*)p; }

__attribute__((visibility("default"))) int oracle_add_elements(void* pp, int energy, int N, int64_t n_elem,
                                                               const int32_t* handles, const double* params, int n_params)
{
    ORACLE_TRY(
        Problem& p = *(Problem*)pp;
        Term t; t.energy = energy; t.N = N; t.n_elem = n_elem; t.n_params = n_params;
        t.handles.assign(handles, handles + n_elem * N);
        t.params.assign(params, params + n_elem * n_params);
        p.terms.push_back(std::move(t));
        p.ldl_ready = false;
        return 0;
    )
}

__attribute__((visibility("default"))) int oracle_eval(void* pp, const double* x, double* f)
{
    ORACLE_TRY(*f = eval(*(Problem*)pp, x); return 0;)
}

__attribute__((visibility("default"))) int oracle_eval_with_gradient(void* pp, const double* x, double* f, double* g)
{
    ORACLE_TRY(
        Problem& p = *(Problem*)pp;
        std::vector<double> gv;
        eval_derivs(p, x, false, false, 0.0, *f, gv);
        std::memcpy(g, gv.data(), sizeof(double) * p.n_vars);
        return 0;
    )
}

// project: 0 = eval_with_derivatives, 1 = eval_with_hessian_proj(eps)
__attribute__((visibility("default"))) int oracle_eval_with_hessian(void* pp, const double* x, int project, double eps,
                                                                    double* f, double* g, int64_t* nnz)
{
    ORACLE_TRY(
        Problem& p = *(Problem*)pp;
        std::vector<double> gv;
        eval_derivs(p, x, true, project != 0, eps, *f, gv);
        std::memcpy(g, gv.data(), sizeof(double) * p.n_vars);
        *nnz = (int64_t)p.values.size();
        return 0;
    )
}

// CSC arrays of the last assembled Hessian
__attribute__((visibility("default"))) int oracle_get_hessian(void* pp, int32_t* outer, int32_t* inner, double* values)
{
    Problem& p = *(Problem*)pp;
    std::memcpy(outer, p.outer.data(), sizeof(int32_t) * p.outer.size());
    std::memcpy(inner, p.inner.data(), sizeof(int32_t) * p.inner.size());
    std::memcpy(values, p.values.data(), sizeof(double) * p.values.size());
    return 0;
}

__attribute__((visibility("default"))) int oracle_newton_direction(void* pp, const double* g, double w, double* d)
{
    ORACLE_TRY(
        Problem& p = *(Problem*)pp;
        std::vector<double> gv(g, g + p.n_vars), dv;
        newton_direction(p, gv, w, dv);
        std::memcpy(d, dv.data(), sizeof(double) * p.n_vars);
        return 0;
    )
}

// returns 0 ok, 4 = line search failed (x unchanged)
__attribute__((visibility("default"))) int oracle_line_search(void* pp, const double* x, const double* d, double f,
                                                              const double* g, double s_max, double* x_out, double* f_out)
{
    ORACLE_TRY(
        Problem& p = *(Problem*)pp;
        std::vector<double> x0(x, x + p.n_vars), dv(d, d + p.n_vars), gv(g, g + p.n_vars), xo;
        const bool ok = line_search(p, x0, dv, f, gv, xo, *f_out, s_max);
        std::memcpy(x_out, xo.data(), sizeof(double) * p.n_vars);
        return ok ? 0 : 4;
    )
}

// Projected Newton (tests/NewtonTest.cc:69-75).  f_hist: n_iters+1 energies.
// times (optional, 4): seconds in [eval+assemble, factor+solve, line search, total].
__attribute__((visibility("default"))) int oracle_newton(void* pp, double* x, int n_iters, double eps,
                                                         double* f_hist, double* times)
{
    ORACLE_TRY(
        Problem& p = *(Problem*)pp;
        std::vector<double> xv(x, x + p.n_vars), g, d, xn;
        double f = 0.0, t_eval = 0, t_solve = 0, t_ls = 0;
        for (int it = 0; it < n_iters; ++it)
        {
            double t0 = omp_get_wtime();
            eval_derivs(p, xv.data(), true, true, eps, f, g);
            double t1 = omp_get_wtime();
            if (f_hist) f_hist[it] = f;
            newton_direction(p, g, 0.0, d);
            double t2 = omp_get_wtime();
            double fn;
            line_search(p, xv, d, f, g, xn, fn);
            xv.swap(xn);
            double t3 = omp_get_wtime();
            t_eval += t1 - t0; t_solve += t2 - t1; t_ls += t3 - t2;
        }
        if (f_hist) f_hist[n_iters] = eval(p, xv.data());
        if (times) { times[0] = t_eval; times[1] = t_solve; times[2] = t_ls; times[3] = t_eval + t_solve + t_ls; }
        std::memcpy(x, xv.data(), sizeof(double) * p.n_vars);
        return 0;
    )
}

// The pattern analysis of the linear solver at x (the Hessian's sparsity and
// the symbolic LDL^T), done once before a solve as the reference's
// LinearSolver caches analyzePattern across iterations (LinearSolver.hh:12-19,
// NewtonDirection.hh:36-41); the timed Newton iterations then only factorise.
__attribute__((visibility("default"))) int oracle_prepare_solver(void* pp, const double* x, double eps)
{
    ORACLE_TRY(
        Problem& p = *(Problem*)pp;
        std::vector<double> g;
        double f = 0.0;
        eval_derivs(p, x, true, true, eps, f, g);
        if (!p.ldl_ready || p.pattern_outer != p.outer || p.pattern_inner != p.inner) ldl_symbolic(p);
        return 0;
    )
}

__attribute__((visibility("default"))) int oracle_n_threads(void* pp) { return get_n_threads(*(Problem*)pp); }

// Univariate operator table (op codes shared with tad_debug_scalar_op):
// a, b = (val, grad, hess) of Scalar<1>; out = (val, grad, hess).
__attribute__((visibility("default"))) int oracle_scalar_op(int op, const double* a3, const double* b3, double* out)
{
    using S = AD<1, double>;
    const S a = S::known(a3[0], a3[1], a3[2]);
    const S b = S::known(b3[0], b3[1], b3[2]);
    S r;
    switch (op)
    {
    case 0: r = -a; break;
    case 1: r = sqrt(a); break;
    case 2: r = sqr(a); break;
    case 3: r = pow(a, (int)b3[0]); break;
    case 4: r = pow(a, b3[0]); break;
    case 5: r = exp(a); break;
    case 6: r = log(a); break;
    case 7: r = sin(a); break;
    case 8: r = cos(a); break;
    case 9: r = tan(a); break;
    case 10: r = asin(a); break;
    case 11: r = acos(a); break;
    case 12: r = atan(a); break;
    case 13: r = sinh(a); break;
    case 14: r = cosh(a); break;
    case 15: r = tanh(a); break;
    case 16: r = fabs(a); break;
    case 17: r = a + b; break;
    case 18: r = a - b; break;
    case 19: r = a * b; break;
    case 20: r = a / b; break;
    case 21: r = atan2(a, b); break;
    case 22: r = hypot(a, b); break;
    case 23: r = b3[0] / a; break;
    case 24: r = log2(a); break;
    case 25: r = log10(a); break;
    case 26: r = asinh(a); break;
    case 27: r = acosh(a); break;
    case 28: r = atanh(a); break;
    case 29: r = a + b3[0]; break;
    case 30: r = a * b3[0]; break;
    case 31: r = b3[0] - a; break;
    case 32: r = a / b3[0]; break;
    default: return 1;
    }
    out[0] = r.val; out[1] = r.grad[0]; out[2] = r.hess[0];
    return 0;
}

} // extern "C"

// Rest-parameterised symmetric Dirichlet of one triangle (UVs a, b, c and 3D
// rest positions Pa, Pb, Pc): the rest edge matrix in the triangle's own
// frame, weight = rest area.
template <typename S>
static S symdir_tri_rest(const std::array<S, 6>& u, const std::array<S, 9>& P)
{
    std::array<S, 3> e, f, n;
    for (int i = 0; i < 3; ++i) { e[i] = P[3 + i] - P[i]; f[i] = P[6 + i] - P[i]; }
    const S l = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    n[0] = e[1] * f[2] - e[2] * f[1];
    n[1] = e[2] * f[0] - e[0] * f[2];
    n[2] = e[0] * f[1] - e[1] * f[0];
    const S an = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    Mat<S, 2, 2> Mr;
    Mr(0, 0) = l; Mr(1, 0) = S(0.0); Mr(0, 1) = (e[0] * f[0] + e[1] * f[1] + e[2] * f[2]) / l; Mr(1, 1) = an / l;
    Mat<S, 2, 2> M;
    M(0, 0) = u[2] - u[0]; M(1, 0) = u[3] - u[1]; M(0, 1) = u[4] - u[0]; M(1, 1) = u[5] - u[1];
    if (value_of(det2(M)) <= 0.0) return S(INFINITY);
    Mat<S, 2, 2> Mri = inv2(Mr), Mi = inv2(M);
    Mat<S, 2, 2> J, K;
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
        {
            J(i, j) = M(i, 0) * Mri(0, j) + M(i, 1) * Mri(1, j);
            K(i, j) = Mr(i, 0) * Mi(0, j) + Mr(i, 1) * Mi(1, j);
        }
    return (squared_norm(J) + squared_norm(K)) * (an * 0.5);
}

extern "C" {

// dL/d(rest) = -(d2E/dx dP)^T lambda with H lambda = dLdx (LDL^T), mixed blocks
// from AD<15> restricted to the x-rows / P-columns block.
__attribute__((visibility("default"))) int oracle_adjoint_rest_gradient(void* pp, const double* x, const double* dLdx,
                                                                        const double* rest, int projected, double eps,
                                                                        double* out, double* lambda)
{
    ORACLE_TRY(
        Problem& p = *(Problem*)pp;
        double f;
        std::vector<double> g;
        eval_derivs(p, x, true, projected != 0, eps, f, g);
        std::vector<double> b(dLdx, dLdx + p.n_vars), lam;
        // newton_direction solves H d = -g: pass -b to get lambda = H^-1 b
        for (double& v : b) v = -v;
        newton_direction(p, b, 0.0, lam);
        if (lambda) std::memcpy(lambda, lam.data(), sizeof(double) * p.n_vars);
        std::fill(out, out + 3 * p.n_handles, 0.0);
        using S = AD<15, double, 0, 6, 6, 9>;
        for (const Term& t : p.terms)
        {
            if (t.energy != TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI) continue;
            for (int64_t e = 0; e < t.n_elem; ++e)
            {
                const int* h = &t.handles[e * 3];
                std::array<S, 6> u;
                std::array<S, 9> P;
                for (int a = 0; a < 3; ++a)
                {
                    for (int i = 0; i < 2; ++i) u[2 * a + i] = S(x[2 * h[a] + i], 2 * a + i);
                    for (int i = 0; i < 3; ++i) P[3 * a + i] = S(rest[3 * h[a] + i], 6 + 3 * a + i);
                }
                const S E = symdir_tri_rest(u, P);
                if (!std::isfinite(E.val)) continue;
                for (int j = 0; j < 9; ++j)
                {
                    double c = 0.0;
                    for (int i = 0; i < 6; ++i) c -= E.H(i, j) * lam[2 * h[i / 2] + (i % 2)];
                    out[3 * h[j / 3] + (j % 3)] += c;
                }
            }
        }
        return 0;
    )
}

} // extern "C"

// Symmetric Dirichlet of one triangle through the truncated-Hessian scalar
// (tests/ScalarTestHessianBlock.cc:50-100): returns the requested block of
// the 6x6 Hessian computed with a full and with a block-restricted scalar.
template <int R0, int C0, int NR, int NC>
static void symdir_block(const double* x6, const double* xr6, double* full, double* blk)
{
    auto energy = [&](auto tag) {
        using S = decltype(tag);
        std::array<S, 6> x;
        for (int i = 0; i < 6; ++i) x[i] = S(x6[i], i);
        Mat<double, 2, 2> Mr;
        Mr(0, 0) = xr6[2] - xr6[0]; Mr(1, 0) = xr6[3] - xr6[1]; Mr(0, 1) = xr6[4] - xr6[0]; Mr(1, 1) = xr6[5] - xr6[1];
        Mat<S, 2, 2> M;
        M(0, 0) = x[2] - x[0]; M(1, 0) = x[3] - x[1]; M(0, 1) = x[4] - x[0]; M(1, 1) = x[5] - x[1];
        const Mat<S, 2, 2> J = matmul(M, inv2(Mr));
        return squared_norm(J) + squared_norm(inv2(J));
    };
    const auto Ef = energy(AD<6, double>());
    const auto Eb = energy(AD<6, double, R0, C0, NR, NC>());
    for (int i = 0; i < NR; ++i)
        for (int j = 0; j < NC; ++j)
        {
            full[i * NC + j] = Ef.H(R0 + i, C0 + j);
            blk[i * NC + j] = Eb.H(i, j);
        }
}

extern "C" {

__attribute__((visibility("default"))) int oracle_symdir_hessian_block(int which, const double* x6, const double* xr6,
                                                                       double* full, double* blk)
{
    switch (which)
    {
    case 0: symdir_block<0, 0, 6, 6>(x6, xr6, full, blk); break;
    case 1: symdir_block<0, 0, 3, 1>(x6, xr6, full, blk); break;
    case 2: symdir_block<0, 0, 1, 3>(x6, xr6, full, blk); break;
    case 3: symdir_block<2, 2, 2, 2>(x6, xr6, full, blk); break;
    case 4: symdir_block<1, 4, 5, 2>(x6, xr6, full, blk); break;
    default: return 1;
    }
    return 0;
}

} // extern "C"
