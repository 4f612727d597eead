/*
 * C++ front-end test (tad/ScalarFunction.cuh): the reference's own test
 * programs written against the drop-in API with generic __device__ lambdas.
 *   planar Newton        tests/NewtonTest.cc:12-95 (nnz formula, f -> 4, g -> 0)
 *   quadratics           tests/ScalarFunctionTest.cc:10-151
 *   element variables    tests/ScalarFunctionTest.cc:153-179 (dedup, too many variables)
 * Prints "frontend ok" and exits 0 on success.
 */
#include <tad/ScalarFunction.cuh>
#include <tad/Mat.cuh>

#include <cmath>
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

int main()
{
    if (planar_newton()) return 1;
    if (quadratics()) return 1;
    if (element_variables()) return 1;
    std::printf("frontend ok\n");
    return 0;
}
