/*
 * C++ front-end test (tad/ScalarFunction.cuh): the reference's own test
 * programs written against the drop-in API with generic __device__ lambdas.
 *   planar Newton        tests/NewtonTest.cc:12-95 (nnz formula, f -> 4, g -> 0)
 *   quadratics           tests/ScalarFunctionTest.cc:10-151
 *   element variables    tests/ScalarFunctionTest.cc:153-179 (dedup, too many variables)
 *   reduced basis        tests/SwitchSolverTest.cc:16-36 (Newton step (-1, -1))
 *   dynamic valences     tests/DynamicElementsTest.cc:9-33 (grouping, term sizes, f/g/H)
 *   vector function      tests/VectorFunctionTest.cc:9-72 (r, J, residual Hessians, sum of squares)
 *   Gauss-Newton         tests/GaussNewtonTest.cc:13-158 (planar mesh, f -> 4)
 *   Laplacian            tests/DynamicElementsTest.cc:35-141 (static triangles and dynamic
 *                        one-ring elements vs the assembled Laplacian, on a closed torus
 *                        with vertex valences 4 and 8)
 * Prints "frontend ok" and exits 0 on success.
 */
#include <tad/ScalarFunction.cuh>
#include <tad/Mat.cuh>

#include <cmath>
#include <algorithm>
#include <cstdio>
#include <vector>

#define CHECK(c)                                                                  \
    do {                                                                          \
        if (!(c)) { std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); return 1; } \
    } while (0)

template <typename T>
static T* to_device(const std::vector<T>& v)
{
    T* p = nullptr;
    tad::check_cuda(cudaMalloc(&p, v.size() * sizeof(T)));
    tad::check_cuda(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return p;
}

static int planar_newton()
{
    // planar_test_mesh (tests/Meshes.hh:12-42)
    const std::vector<double> V_rest = {0, 0, 1, 0, 0, 1, 1, 1, 0, 2, 1, 2};
    std::vector<double> V = V_rest;
    for (int v = 0; v < 6; ++v) { V[2 * v] *= 0.5; V[2 * v + 1] *= 0.25; }
    const std::vector<int> F = {0, 1, 2, 1, 3, 2, 2, 3, 5, 2, 5, 4};
    const std::vector<int> b = {0, 4};
    const std::vector<double> bc = {0.0, 0.0, -2.0, 0.0};
    const double* Vr = to_device(V_rest);
    const int* Fd = to_device(F);
    const int* bd = to_device(b);
    const double* bcd = to_device(bc);
    const int nF = 4;

    auto func = tad::scalar_function<2>(tad::range(6));
    func.add_elements<3>(tad::range(nF), [=] __device__(auto& element) {
        using T = TAD_SCALAR_TYPE(element);
        using P = TAD_PASSIVE_TYPE(element);
        const int f = (int)element.handle;
        tad::Vec<P, 2> ar, br, cr;
        for (int i = 0; i < 2; ++i)
        {
            ar[i] = (P)Vr[2 * Fd[3 * f + 0] + i];
            br[i] = (P)Vr[2 * Fd[3 * f + 1] + i];
            cr[i] = (P)Vr[2 * Fd[3 * f + 2] + i];
        }
        const tad::Mat<P, 2, 2> Mr = tad::col_mat(br - ar, cr - ar);
        const tad::Vec<T, 2> a = element.variables(Fd[3 * f + 0]);
        const tad::Vec<T, 2> bb = element.variables(Fd[3 * f + 1]);
        const tad::Vec<T, 2> c = element.variables(Fd[3 * f + 2]);
        const tad::Mat<T, 2, 2> M = tad::col_mat(bb - a, c - a);
        if (tad::determinant(M) <= 0.0) return T(INFINITY);
        return ((M * tad::inverse(Mr)).squaredNorm() + (Mr * tad::inverse(M)).squaredNorm()) / (P)nF;
    });
    func.add_elements<1>(tad::range(2), [=] __device__(auto& element) {
        using T = TAD_SCALAR_TYPE(element);
        using P = TAD_PASSIVE_TYPE(element);
        const int h = (int)element.handle;
        tad::Vec<P, 2> target;
        target[0] = (P)bcd[2 * h];
        target[1] = (P)bcd[2 * h + 1];
        const tad::Vec<T, 2> p = element.variables(bd[h]);
        return (target - p).squaredNorm();
    });
    std::vector<double> x = func.x_from_data([&](int64_t v) { return std::array<double, 2>{V[2 * v], V[2 * v + 1]}; });
    {
        auto [f, g, H] = func.eval_with_hessian_proj(x);
        CHECK(H.nonZeros() == 4 * 6 + 8 * (6 + 4 - 1));
        (void)f; (void)g;
    }
    for (int i = 0; i < 10; ++i)
    {
        auto [f, g, H] = func.eval_with_hessian_proj(x);
        const std::vector<double> d = func.newton_direction(x);
        // the stopping test of the reference's loops (NewtonDecrement.hh:20-26)
        const double dec = func.newton_decrement(d, g);
        double ref = 0.0;
        for (size_t j = 0; j < d.size(); ++j) ref += d[j] * g[j];
        ref *= -0.5;
        CHECK(std::fabs(dec - ref) <= 1e-12 * std::fabs(ref) + 1e-300);
        if (dec < 1e-24) break;
        x = func.line_search(x, d, f, g);
        (void)H;
    }
    auto [f, g, H] = func.eval_with_hessian_proj(x);
    double gmax = 0.0;
    for (double v : g) gmax = std::fmax(gmax, std::fabs(v));
    std::printf("planar newton: f = %.17g, |g|max = %.3g\n", f, gmax);
    CHECK(std::fabs(func.eval(x) - f) <= 1e-15);
    CHECK(std::fabs(f - 4.0) <= 1e-12);
    CHECK(gmax <= 1e-10);
    // fused device loop reaches the same minimum
    std::vector<double> x2 = func.newton_solve(func.x_from_data([&](int64_t v) { return std::array<double, 2>{V[2 * v], V[2 * v + 1]}; }), 10);
    CHECK(std::fabs(func.eval(x2) - 4.0) <= 1e-12);
    return 0;
}

static int quadratics()
{
    auto func = tad::scalar_function<2>(tad::range(1));
    func.add_elements<1>(tad::range(1), [] __device__(auto& element) {
        const auto v = element.variables(0);
        return 2.0 * tad::sqr(v[0]) + 2.0 * v[0] * v[1] + tad::sqr(v[1]) + v[0] + 1.0;
    });
    const std::vector<double> x = {1.0, 2.0};
    auto [f, g, H] = func.eval_with_derivatives(x);
    CHECK(f == 12.0 && g[0] == 9.0 && g[1] == 6.0);
    CHECK(H.coeff(0, 0) == 4.0 && H.coeff(0, 1) == 2.0 && H.coeff(1, 0) == 2.0 && H.coeff(1, 1) == 2.0);
    auto [f2, g2, H2] = func.eval_with_hessian_proj(x);
    CHECK(f2 == 12.0 && H2.coeff(0, 0) == 4.0 && H2.coeff(1, 1) == 2.0);
    auto [fg, gg] = func.eval_with_gradient(x);
    CHECK(fg == 12.0 && gg[0] == 9.0 && gg[1] == 6.0);

    // SwitchSolverTest.cc:16-36: x^2 + y^2 at (1, 1), B = I: Newton step (-1, -1)
    auto circ = tad::scalar_function<2>(tad::range(1));
    circ.add_elements<1>(tad::range(1), [] __device__(auto& element) {
        const auto v = element.variables(0);
        return tad::sqr(v[0]) + tad::sqr(v[1]);
    });
    tad::SparseCSR B;
    B.rows = 2;
    B.outer = {0, 1, 2};
    B.inner = {0, 1};
    B.values = {1.0, 1.0};
    const std::vector<double> dr = circ.newton_direction_reduced_basis({1.0, 1.0}, B, 2);
    CHECK(std::fabs(dr[0] + 1.0) <= 1e-15 && std::fabs(dr[1] + 1.0) <= 1e-15);
    const std::vector<double> dn = circ.newton_direction({1.0, 1.0});
    CHECK(std::fabs(dn[0] + 1.0) <= 1e-15 && std::fabs(dn[1] + 1.0) <= 1e-15);

    auto neg = tad::scalar_function<2>(tad::range(1));
    neg.add_elements<1>(tad::range(1), [] __device__(auto& element) {
        const auto v = element.variables(0);
        return -(2.0 * tad::sqr(v[0]) + 2.0 * v[0] * v[1] + tad::sqr(v[1]) + v[0] + 1.0);
    });
    auto [fn, gn, Hp] = neg.eval_with_hessian_proj(x);
    const double a = Hp.coeff(0, 0), bq = Hp.coeff(0, 1), c = Hp.coeff(1, 1);
    CHECK(fn == -12.0 && a > 0.0 && a * c - bq * bq > 0.0);   // positive definite
    return 0;
}

static int element_variables()
{
    // variables(0) twice: deduplicated, identical seeds (ScalarFunctionTest.cc:153-179)
    auto func = tad::scalar_function<2>(tad::range(2));
    func.add_elements<1>(tad::range(1), [] __device__(auto& element) {
        using T = TAD_SCALAR_TYPE(element);
        const auto v = element.variables(0);
        const auto v2 = element.variables(0);
        return (v[0] - v2[0]) * (v[1] - v2[1]) + T(0.0);
    });
    auto [f, g, H] = func.eval_with_hessian_proj(std::vector<double>(4, 0.0));
    CHECK(f == 0.0);
    // more handles than the valence: the reference throws "Too many variables requested"
    auto bad = tad::scalar_function<2>(tad::range(2));
    bad.add_elements<1>(tad::range(1), [] __device__(auto& element) {
        const auto v = element.variables(0);
        const auto w = element.variables(1);
        return v[0] * w[0];
    });
    bool threw = false;
    try { bad.eval(std::vector<double>(4, 1.0)); }
    catch (const std::runtime_error& e) { threw = std::string(e.what()).find("Too many variables") != std::string::npos; }
    CHECK(threw);
    return 0;
}

static int dynamic_valences()
{
    // element e accesses variables 0..e-1 and returns |sum|^2; valences <3, 1>
    auto func = tad::scalar_function<2>(tad::range(4));
    func.add_elements_dynamic<3, 1>(tad::range(4), [] __device__(auto& element) {
        using T = TAD_SCALAR_TYPE(element);
        const int e = (int)element.handle;
        tad::Vec<T, 2> sum;
        sum[0] = T(0.0);
        sum[1] = T(0.0);
        for (int v = 0; v < e; ++v) sum = sum + element.variables(v);
        return sum.squaredNorm();
    });
    CHECK(func.n_terms() == 2);
    CHECK(func.term_n_elements(0) == 2 && func.term_n_elements(1) == 2);
    auto [f, g, H] = func.eval_with_hessian_proj(std::vector<double>(8, 1.0));
    // f = sum_e 2 e^2; g_v = 2 sum_{e > v} (e, e); H(v, w) = 2 (3 - max(v, w)) I for max(v, w) < 3
    CHECK(f == 28.0);
    const double gx[4] = {12.0, 10.0, 6.0, 0.0};
    for (int v = 0; v < 4; ++v) CHECK(g[2 * v] == gx[v] && g[2 * v + 1] == gx[v]);
    for (int v = 0; v < 3; ++v)
        for (int w = 0; w < 3; ++w)
        {
            const double ex = 2.0 * (3 - std::max(v, w));
            CHECK(std::fabs(H.coeff(2 * v, 2 * w) - ex) <= 1e-8 && std::fabs(H.coeff(2 * v + 1, 2 * w + 1) - ex) <= 1e-8);
            CHECK(std::fabs(H.coeff(2 * v, 2 * w + 1)) <= 1e-8);
        }
    // a valence above every listed one is an error (ScalarFunctionImpl.hh:185-190)
    auto small = tad::scalar_function<2>(tad::range(4));
    bool threw = false;
    try
    {
        small.add_elements_dynamic<2, 1>(tad::range(4), [] __device__(auto& element) {
            using T = TAD_SCALAR_TYPE(element);
            const int e = (int)element.handle;
            T acc = T(0.0);
            for (int v = 0; v < e; ++v) acc = acc + element.variables(v)[0];
            return acc * acc;
        });
    }
    catch (const std::runtime_error&) { threw = true; }
    CHECK(threw);
    return 0;
}

static int dynamic_laplacian()
{
    // closed torus, nu x nv grid, quads split along alternating diagonals:
    // vertex valences 4 and 8 (one-ring elements of 5 and 9 handles)
    const int nu = 8, nv = 6, nV = nu * nv;
    auto vid = [&](int i, int j) { return ((i + nu) % nu) * nv + (j + nv) % nv; };
    std::vector<int> F;
    for (int i = 0; i < nu; ++i)
        for (int j = 0; j < nv; ++j)
        {
            const int a = vid(i, j), b = vid(i + 1, j), c = vid(i + 1, j + 1), dd = vid(i, j + 1);
            if ((i + j) % 2 == 0) { F.insert(F.end(), {a, b, c, a, c, dd}); }
            else { F.insert(F.end(), {a, b, dd, b, c, dd}); }
        }
    const int nF = (int)F.size() / 3;
    // reference Laplacian of the directed face edges (DynamicElementsTest.cc:38-55)
    std::vector<double> L(nV * nV, 0.0);
    std::vector<std::vector<int>> nbr(nV);
    for (int f = 0; f < nF; ++f)
        for (int i = 0; i < 3; ++i)
        {
            const int v1 = F[3 * f + i], v2 = F[3 * f + (i + 1) % 3];
            L[v1 * nV + v1] += 1.0;
            L[v1 * nV + v2] -= 1.0;
            nbr[v1].push_back(v2);
        }
    std::vector<int> nptr(nV + 1, 0), nidx;
    for (int v = 0; v < nV; ++v) { nptr[v + 1] = nptr[v] + (int)nbr[v].size(); nidx.insert(nidx.end(), nbr[v].begin(), nbr[v].end()); }
    const int* Fd = to_device(F);
    const int* np = to_device(nptr);
    const int* ni = to_device(nidx);
    auto dense = [&](const tad::SparseCSR& H) {
        std::vector<double> D(nV * nV, 0.0);
        for (int r = 0; r < nV; ++r)
            for (int q = H.outer[r]; q < H.outer[r + 1]; ++q) D[r * nV + H.inner[q]] += H.values[q];
        return D;
    };
    auto err_to_ref = [&](const std::vector<double>& D) {
        double e2 = 0.0;
        for (int i = 0; i < nV * nV; ++i) e2 += (D[i] - 0.5 * (L[i] + L[(i % nV) * nV + i / nV])) * (D[i] - 0.5 * (L[i] + L[(i % nV) * nV + i / nV]));
        return std::sqrt(e2);
    };
    int ref_nnz = 0;
    for (int i = 0; i < nV * nV; ++i) ref_nnz += (L[i] != 0.0 || L[(i % nV) * nV + i / nV] != 0.0) ? 1 : 0;

    // static triangle elements
    auto tri = tad::scalar_function<1>(tad::range(nV));
    tri.add_elements<3>(tad::range(nF), [=] __device__(auto& element) {
        const int f = (int)element.handle;
        const auto a = element.variable(Fd[3 * f + 0]);
        const auto b = element.variable(Fd[3 * f + 1]);
        const auto c = element.variable(Fd[3 * f + 2]);
        return 0.25 * (tad::sqr(b - a) + tad::sqr(c - b) + tad::sqr(a - c));
    });
    const tad::SparseCSR Ht = tri.eval_hessian_of_quadratic();
    const double et = err_to_ref(dense(Ht));
    std::printf("laplacian (triangles): |L - L_ref| = %.3g, nnz %lld vs %d\n", et, (long long)Ht.nonZeros(), ref_nnz);
    CHECK(et <= 1e-12);
    CHECK(Ht.nonZeros() == ref_nnz);

    // dynamic one-ring vertex elements: valences 5 and 9 go to the groups 6 and 10
    auto ring = tad::scalar_function<1>(tad::range(nV));
    ring.add_elements_dynamic<6, 10>(tad::range(nV), [=] __device__(auto& element) {
        using T = TAD_SCALAR_TYPE(element);
        const int v = (int)element.handle;
        const T vv = element.variable(v);
        T dirichlet = T(0.0);
        for (int q = np[v]; q < np[v + 1]; ++q) dirichlet = dirichlet + 0.25 * tad::sqr(vv - element.variable(ni[q]));
        return dirichlet;
    });
    CHECK(ring.n_terms() == 2);
    int n5 = 0;
    for (int v = 0; v < nV; ++v) n5 += nbr[v].size() == 4 ? 1 : 0;
    CHECK(ring.term_n_elements(0) == n5 && ring.term_n_elements(1) == nV - n5);
    const double er = err_to_ref(dense(ring.eval_hessian_of_quadratic()));
    std::printf("laplacian (one-ring dynamic): |L - L_ref| = %.3g\n", er);
    CHECK(er <= 1e-12);
    return 0;
}

static int vector_function_basic()
{
    // R^2 -> R^3: element 1 gives (2 x0, x0^2), element 2 gives (x1^2)
    auto func = tad::vector_function<1>(tad::range(2));
    func.add_elements<1, 2>(tad::range(1), [] __device__(auto& element) {
        using T = TAD_SCALAR_TYPE(element);
        const T x0 = element.variables(0)[0];
        tad::Vec<T, 2> r;
        r[0] = 2.0 * x0;
        r[1] = tad::sqr(x0);
        return r;
    });
    func.add_elements<1, 1>(tad::range(1), [] __device__(auto& element) {
        using T = TAD_SCALAR_TYPE(element);
        const T x1 = element.variables(1)[0];
        tad::Vec<T, 1> r;
        r[0] = tad::sqr(x1);
        return r;
    });
    const std::vector<double> x = {3.0, 4.0};
    const std::vector<double> r = func.eval(x);
    CHECK(r.size() == 3 && r[0] == 6.0 && r[1] == 9.0 && r[2] == 16.0);
    CHECK(func.eval_sum_of_squares(x) == 373.0);
    auto [f, g, rs, Js] = func.eval_sum_of_squares_with_derivatives(x);
    CHECK(f == 373.0 && rs[2] == 16.0);
    CHECK(g[0] == 8.0 * x[0] + 4.0 * x[0] * x[0] * x[0] && g[1] == 4.0 * x[1] * x[1] * x[1]);
    auto [rj, J] = func.eval_with_jacobian(x);
    CHECK(J.rows == 3 && J.cols == 2);
    CHECK(J.coeff(0, 0) == 2.0 && J.coeff(1, 0) == 6.0 && J.coeff(2, 1) == 8.0 && J.coeff(0, 1) == 0.0);
    auto [rh, Jh, H] = func.eval_with_derivatives(x);
    CHECK(H.size() == 3);
    CHECK(H[0].coeff(0, 0) == 0.0 && H[1].coeff(0, 0) == 2.0 && H[2].coeff(1, 1) == 2.0);
    return 0;
}

static int gauss_newton_planar()
{
    // tests/GaussNewtonTest.cc: symmetric Dirichlet residuals (8 per triangle)
    // and position residuals, 20 Gauss-Newton steps with w = 1e-12
    const std::vector<double> V_rest = {0, 0, 1, 0, 0, 1, 1, 1, 0, 2, 1, 2};
    std::vector<double> V = V_rest;
    for (int v = 0; v < 6; ++v) { V[2 * v] *= 0.5; V[2 * v + 1] *= 0.25; }
    const std::vector<int> F = {0, 1, 2, 1, 3, 2, 2, 3, 5, 2, 5, 4};
    const std::vector<int> b = {0, 4};
    const std::vector<double> bc = {0.0, 0.0, -2.0, 0.0};
    const double* Vr = to_device(V_rest);
    const int* Fd = to_device(F);
    const int* bd = to_device(b);
    const double* bcd = to_device(bc);
    const int nF = 4;
    tad_settings st;
    tad_settings_default(&st);
    st.pcg_rel_tol = 1e-12;
    auto func = tad::vector_function<2>(tad::range(6), &st);
    func.add_elements<3, 8>(tad::range(nF), [=] __device__(auto& element) {
        using T = TAD_SCALAR_TYPE(element);
        using P = TAD_PASSIVE_TYPE(element);
        const int f = (int)element.handle;
        tad::Vec<P, 2> ar, br, cr;
        for (int i = 0; i < 2; ++i)
        {
            ar[i] = (P)Vr[2 * Fd[3 * f + 0] + i];
            br[i] = (P)Vr[2 * Fd[3 * f + 1] + i];
            cr[i] = (P)Vr[2 * Fd[3 * f + 2] + i];
        }
        const tad::Mat<P, 2, 2> Mr = tad::col_mat(br - ar, cr - ar);
        const tad::Vec<T, 2> a = element.variables(Fd[3 * f + 0]);
        const tad::Vec<T, 2> bb = element.variables(Fd[3 * f + 1]);
        const tad::Vec<T, 2> c = element.variables(Fd[3 * f + 2]);
        const tad::Mat<T, 2, 2> M = tad::col_mat(bb - a, c - a);
        tad::Vec<T, 8> E;
        if (tad::determinant(M) <= 0.0)
        {
            for (int o = 0; o < 8; ++o) E[o] = T(INFINITY);
            return E;
        }
        const tad::Mat<T, 2, 2> J = M * tad::inverse(Mr);
        const tad::Mat<T, 2, 2> Ji = Mr * tad::inverse(M);
        const P s = P(1.0 / sqrt((double)nF));
        E[0] = J(0, 0) * s; E[1] = J(0, 1) * s; E[2] = J(1, 0) * s; E[3] = J(1, 1) * s;
        E[4] = Ji(0, 0) * s; E[5] = Ji(0, 1) * s; E[6] = Ji(1, 0) * s; E[7] = Ji(1, 1) * s;
        return E;
    });
    func.add_elements<1, 2>(tad::range(2), [=] __device__(auto& element) {
        using T = TAD_SCALAR_TYPE(element);
        using P = TAD_PASSIVE_TYPE(element);
        const int h = (int)element.handle;
        const tad::Vec<T, 2> p = element.variables(bd[h]);
        tad::Vec<T, 2> r;
        r[0] = P(bcd[2 * h]) - p[0];
        r[1] = P(bcd[2 * h + 1]) - p[1];
        return r;
    });
    CHECK(func.n_outputs() == 4 * 8 + 2 * 2);
    std::vector<double> x = func.x_from_data([&](int64_t v) { return std::array<double, 2>{V[2 * v], V[2 * v + 1]}; });
    for (int i = 0; i < 20; ++i)
    {
        auto [f, g, r, J] = func.eval_sum_of_squares_with_derivatives(x);
        const std::vector<double> d = func.gauss_newton_direction(x, 1e-12);
        x = func.line_search(x, d, f, g);
    }
    auto [f, g, r, J] = func.eval_sum_of_squares_with_derivatives(x);
    double gmax = 0.0;
    for (double v : g) gmax = std::fmax(gmax, std::fabs(v));
    std::printf("gauss-newton planar: f = %.12g, |g|max = %.3g\n", f, gmax);
    CHECK(std::fabs(f - 4.0) <= 0.1 && gmax <= 0.1);
    return 0;
}

int main()
{
    if (planar_newton()) return 1;
    if (quadratics()) return 1;
    if (element_variables()) return 1;
    if (dynamic_valences()) return 1;
    if (dynamic_laplacian()) return 1;
    if (vector_function_basic()) return 1;
    if (gauss_newton_planar()) return 1;
    std::printf("frontend ok\n");
    return 0;
}
