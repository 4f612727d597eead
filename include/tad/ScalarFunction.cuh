/*
 * tad/ScalarFunction.cuh -- C++17 front end with TinyAD's spelling:
 *
 *   auto func = tad::scalar_function<2>(tad::range(n_vertices));
 *   func.add_elements<3>(tad::range(n_faces), [=] __device__ (auto& element) {
 *       using T = TAD_SCALAR_TYPE(element);
 *       ...
 *       if (det <= 0.0) return T(INFINITY);
 *       return energy;                       // every branch returns a T
 *   });
 *   auto [f, g, H] = func.eval_with_hessian_proj(x);
 *
 * (include/TinyAD/ScalarFunction.hh:57-248, Detail/ScalarFunctionImpl.hh).
 * The element functor runs on the device only: a generic __device__ lambda
 * (nvcc --extended-lambda) or a struct with a templated operator(),
 * capturing device pointers and PODs.  Two nvcc limits shape the lambda
 * form: generic __host__ __device__ extended lambdas are rejected, and a
 * trailing return type that depends on the generic parameter (the
 * reference's `-> TINYAD_SCALAR_TYPE(element)`) breaks nvcc's host stub, so
 * the lambda deduces its return type and every branch returns T(...).  It is instantiated here, in the user's
 * translation unit, by the kernels of tad/ElementKernels.cuh and handed to
 * the library (libtad.so, include/tad.h) as a term callback; the library
 * records each element's first-access handle order once, builds the sparsity
 * pattern and runs assembly, PCG and line search.  Results come back in host
 * std::vectors; the Hessian as CSR arrays (identical to Eigen's CSC arrays
 * for the symmetric H).  Errors throw std::runtime_error as the reference's
 * TINYAD_ERROR_throw does.
 */
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <map>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "../tad.h"
#include "ElementKernels.cuh"

namespace tad {

inline void check(tad_status s)
{
    if (s != TAD_OK) throw std::runtime_error(tad_last_error_message());
}

inline void check_cuda(cudaError_t e)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(e));
}

/* TinyAD::range(n) (include/TinyAD/Utils/Helpers.hh:17-27) */
struct IndexRange
{
    int64_t n;
    struct It
    {
        int64_t i;
        int64_t operator*() const { return i; }
        It& operator++() { ++i; return *this; }
        bool operator!=(const It& o) const { return i != o.i; }
    };
    It begin() const { return {0}; }
    It end() const { return {n}; }
    int64_t size() const { return n; }
};
inline IndexRange range(int64_t n) { return {n}; }

/* sparse matrix returned by the eval functions: CSR (== CSC of the symmetric H) */
struct SparseCSR
{
    int64_t rows = 0;
    int64_t cols = 0;        // 0: square (rows x rows)
    std::vector<int32_t> outer, inner;
    std::vector<double> values;
    int64_t nonZeros() const { return (int64_t)values.size(); }
    double coeff(int64_t r, int64_t c) const
    {
        for (int32_t q = outer[r]; q < outer[r + 1]; ++q)
            if (inner[q] == c) return values[q];
        return 0.0;
    }
};

namespace detail {

struct TermBase
{
    virtual ~TermBase() = default;
    virtual int launch(const tad_term_eval_args* a) = 0;
};

/* passes the user's element handle (from the range) instead of the index */
template <typename F>
struct HandleMapped
{
    F f;
    const int32_t* handles;
    template <typename El>
    __device__ auto operator()(El& element) const
    {
        const int64_t e = element.handle;
        element.handle = handles[e];
        auto r = f(element);
        element.handle = e;
        return r;
    }
};

template <int d, int N, typename F>
struct Term : TermBase
{
    HandleMapped<F> fn;
    explicit Term(HandleMapped<F> f) : fn(std::move(f)) {}
    int launch(const tad_term_eval_args* a) override
    {
        tad::launch_elements<d, N>(a->mode, a->precision, make_launch(*a), fn, (cudaStream_t)a->stream);
        return cudaGetLastError() == cudaSuccess ? 0 : 1;
    }
};

template <int d, int N, int M, typename F>
struct VecTerm : TermBase
{
    HandleMapped<F> fn;
    explicit VecTerm(HandleMapped<F> f) : fn(std::move(f)) {}
    int launch(const tad_term_eval_args* a) override
    {
        tad::launch_vector_elements<d, N, M>(a->mode, a->precision, make_launch(*a), fn, (cudaStream_t)a->stream);
        return cudaGetLastError() == cudaSuccess ? 0 : 1;
    }
};

inline int term_callback(void* user, const tad_term_eval_args* a)
{
    try { return static_cast<TermBase*>(user)->launch(a); }
    catch (...) { return 1; }
}

} // namespace detail

template <int d>
class ScalarFunction
{
public:
    using VecD = std::array<double, d>;

    explicit ScalarFunction(int64_t n_handles, const tad_settings* settings = nullptr) : n_handles_(n_handles)
    {
        check(tad_problem_create(d, n_handles, settings, &p_));
    }
    ~ScalarFunction()
    {
        if (p_) tad_problem_destroy(p_);
        for (int32_t* h : handle_bufs_) cudaFree(h);
    }
    ScalarFunction(const ScalarFunction&) = delete;
    ScalarFunction& operator=(const ScalarFunction&) = delete;
    ScalarFunction(ScalarFunction&& o) noexcept { swap(o); }
    ScalarFunction& operator=(ScalarFunction&& o) noexcept { swap(o); return *this; }

    int64_t n_vars() const { return d * n_handles_; }
    tad_problem* handle() { return p_; }

    /* add_elements<N>(range, functor) (ScalarFunctionImpl.hh:63-100) */
    template <int N, typename Range, typename F>
    void add_elements(const Range& elements, F functor)
    {
        std::vector<int32_t> h;
        for (auto eh : elements) h.push_back((int32_t)eh);
        int32_t* hd = nullptr;
        check_cuda(cudaMalloc(&hd, std::max<size_t>(h.size(), 1) * sizeof(int32_t)));
        handle_bufs_.push_back(hd);
        if (!h.empty()) check_cuda(cudaMemcpy(hd, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
        auto term = std::make_unique<detail::Term<d, N, F>>(detail::HandleMapped<F>{functor, hd});
        check(tad_add_elements_custom(p_, N, (int64_t)h.size(), &detail::term_callback, term.get()));
        terms_.push_back(std::move(term));
        term_sizes_.push_back((int64_t)h.size());
    }

    /* add_elements_dynamic<V...>(range, functor) (ScalarFunctionImpl.hh:133-214):
       every element's distinct accessed handles are counted once on the
       device (the functor run with x = 0, as the reference's recorder
       element does), the element joins the smallest listed valence that
       holds it, and one term per non-empty group is added in the order the
       valences are listed -- so the functor is instantiated once per
       valence, each group runs its own element kernels. */
    template <int... Valences, typename Range, typename F>
    void add_elements_dynamic(const Range& elements, F functor)
    {
        static_assert(sizeof...(Valences) >= 1, "At least one element valence has to be passed.");
        static_assert(((Valences >= 1) && ...), "Element valences must be positive.");
        constexpr int vmax = std::max({Valences...});
        std::vector<int> sorted = {Valences...};
        std::sort(sorted.begin(), sorted.end());
        if (std::unique(sorted.begin(), sorted.end()) != sorted.end())
            throw std::runtime_error("Element valences passed to add_elements<..>(..) are not unique. Please pass unique element valences.");
        std::vector<int32_t> h;
        for (auto eh : elements) h.push_back((int32_t)eh);
        const std::vector<int> counts = record_valences<vmax>(h, functor);
        std::map<int, std::vector<int32_t>> groups;
        for (size_t i = 0; i < h.size(); ++i)
        {
            const auto it = std::lower_bound(sorted.begin(), sorted.end(), counts[i]);
            if (it == sorted.end())
                throw std::runtime_error("Element valence " + std::to_string(counts[i]) +
                                         " Exceeds maximum static valence passed to add_elements<..>(..).");
            groups[*it].push_back(h[i]);
        }
        (add_group<Valences>(groups, functor), ...);
    }

    /* number of terms and their element counts (the reference's
       objective_terms[i]->n_elements()) */
    size_t n_terms() const { return term_sizes_.size(); }
    int64_t term_n_elements(size_t i) const { return term_sizes_.at(i); }

    /* x_from_data / x_to_data (ScalarFunctionImpl.hh:216-254) */
    std::vector<double> x_from_data(const std::function<VecD(int64_t)>& read) const
    {
        std::vector<double> x(n_vars());
        for (int64_t v = 0; v < n_handles_; ++v)
        {
            const VecD p = read(v);
            for (int i = 0; i < d; ++i) x[d * v + i] = p[i];
        }
        return x;
    }
    void x_to_data(const std::vector<double>& x, const std::function<void(int64_t, const VecD&)>& write) const
    {
        for (int64_t v = 0; v < n_handles_; ++v)
        {
            VecD p;
            for (int i = 0; i < d; ++i) p[i] = x[d * v + i];
            write(v, p);
        }
    }

    double eval(const std::vector<double>& x) const
    {
        double f;
        check(tad_eval(p_, x.data(), &f));
        return f;
    }
    double operator()(const std::vector<double>& x) const { return eval(x); }

    std::tuple<double, std::vector<double>> eval_with_gradient(const std::vector<double>& x) const
    {
        double f;
        std::vector<double> g(n_vars());
        check(tad_eval_with_gradient(p_, x.data(), &f, g.data()));
        return {f, std::move(g)};
    }

    std::tuple<double, std::vector<double>, SparseCSR> eval_with_derivatives(const std::vector<double>& x) const
    {
        double f;
        std::vector<double> g(n_vars());
        SparseCSR H = pattern();
        check(tad_eval_with_derivatives(p_, x.data(), &f, g.data(), H.values.data()));
        return {f, std::move(g), std::move(H)};
    }

    SparseCSR eval_hessian(const std::vector<double>& x) const { return std::get<2>(eval_with_derivatives(x)); }

    /* the Hessian at x = 0 (ScalarFunctionImpl.hh:370-376) */
    SparseCSR eval_hessian_of_quadratic() const { return eval_hessian(std::vector<double>(n_vars(), 0.0)); }

    std::tuple<double, std::vector<double>, SparseCSR>
    eval_with_hessian_proj(const std::vector<double>& x, double projection_eps = 1e-9) const
    {
        double f;
        std::vector<double> g(n_vars());
        SparseCSR H = pattern();
        check(tad_eval_with_hessian_proj(p_, x.data(), projection_eps, &f, g.data(), H.values.data()));
        return {f, std::move(g), std::move(H)};
    }

    /* newton_direction(g, H_proj, solver) at x (NewtonDirection.hh:25-65) */
    std::vector<double> newton_direction(const std::vector<double>& x, double projection_eps = 1e-9) const
    {
        std::vector<double> dvec(n_vars()), g(n_vars());
        double f;
        const tad_status s = tad_newton_direction(p_, x.data(), 1, projection_eps, 0.0, dvec.data(), &f, g.data());
        if (s != TAD_OK && s != TAD_ERR_PCG_NOCONV) check(s);
        return dvec;
    }

    /* newton_direction_reduced_basis(g, H_proj, B, solver, w) at x
       (NewtonDirection.hh:76-123): d = B (B^T H B + w I)^-1 (-B^T g), B the
       n_vars x m basis in CSR */
    std::vector<double> newton_direction_reduced_basis(const std::vector<double>& x, const SparseCSR& B, int64_t m,
                                                       double w_identity = 0.0, double projection_eps = 1e-9) const
    {
        if (B.rows != n_vars() || (int64_t)B.outer.size() != n_vars() + 1)
            throw std::runtime_error("basis must have n_vars rows");
        std::vector<double> dvec(n_vars()), g(n_vars());
        double f;
        const tad_status s = tad_newton_direction_reduced_basis(p_, x.data(), m, B.outer.data(), B.inner.data(),
                                                                B.values.data(), projection_eps, w_identity,
                                                                dvec.data(), &f, g.data());
        if (s != TAD_OK && s != TAD_ERR_PCG_NOCONV) check(s);
        return dvec;
    }

    /* newton_decrement(d, g) = -d.g / 2 (NewtonDecrement.hh:20-26), the
       usual stopping test of a Newton loop */
    double newton_decrement(const std::vector<double>& dvec, const std::vector<double>& g) const
    {
        if ((int64_t)dvec.size() != n_vars() || (int64_t)g.size() != n_vars())
            throw std::runtime_error("d and g must hold n_vars values");
        double out = 0.0;
        check(tad_newton_decrement(p_, dvec.data(), g.data(), &out));
        return out;
    }

    /* line_search(x0, d, f, g, func) (LineSearch.hh:26-65) */
    std::vector<double> line_search(const std::vector<double>& x0, const std::vector<double>& dvec, double f,
                                    const std::vector<double>& g, double s_max = 1.0) const
    {
        std::vector<double> x(n_vars());
        double fo;
        const tad_status s = tad_line_search(p_, x0.data(), dvec.data(), f, g.data(), s_max, x.data(), &fo);
        if (s != TAD_OK && s != TAD_ERR_LS_FAIL) check(s);
        return x;
    }

    /* the Projected-Newton loop, fused on the device */
    std::vector<double> newton_solve(std::vector<double> x, int iters, double projection_eps = 1e-9) const
    {
        int done = 0;
        check(tad_newton_solve(p_, x.data(), iters, projection_eps, 0.0, nullptr, &done));
        return x;
    }

protected:
    int32_t* upload_handles(const std::vector<int32_t>& h)
    {
        int32_t* hd = nullptr;
        check_cuda(cudaMalloc(&hd, std::max<size_t>(h.size(), 1) * sizeof(int32_t)));
        handle_bufs_.push_back(hd);
        if (!h.empty()) check_cuda(cudaMemcpy(hd, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
        return hd;
    }

    /* distinct accessed handles per element, recorded on the device with the
       functor evaluated at x = 0 and at most vmax handles an element */
    template <int vmax, typename F>
    std::vector<int> record_valences(const std::vector<int32_t>& h, F& functor)
    {
        const int64_t n = (int64_t)h.size();
        std::vector<int> counts(n, 0);
        if (n == 0) return counts;
        void* sp = nullptr;
        check(tad_get_stream(p_, &sp));
        cudaStream_t st = (cudaStream_t)sp;
        int32_t *hd = nullptr, *rec = nullptr, *err = nullptr;
        double* xz = nullptr;
        check_cuda(cudaMalloc(&hd, n * sizeof(int32_t)));
        check_cuda(cudaMalloc(&rec, n * vmax * sizeof(int32_t)));
        check_cuda(cudaMalloc(&err, sizeof(int32_t)));
        check_cuda(cudaMalloc(&xz, std::max<int64_t>(n_vars(), 1) * sizeof(double)));
        std::vector<int32_t> rec_h(n * vmax);
        int32_t err_h = 0;
        check_cuda(cudaMemcpyAsync(hd, h.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
        check_cuda(cudaMemsetAsync(xz, 0, std::max<int64_t>(n_vars(), 1) * sizeof(double), st));
        check_cuda(cudaMemsetAsync(err, 0, sizeof(int32_t), st));
        ElemLaunch L{};
        L.n_elem = n;
        L.x = xz;
        L.record = rec;
        L.err = err;
        k_elem_record<d, vmax, detail::HandleMapped<F>><<<elem_grid(n), 128, 0, st>>>(L, detail::HandleMapped<F>{functor, hd});
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(rec_h.data(), rec, n * vmax * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&err_h, err, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        cudaFree(hd); cudaFree(rec); cudaFree(err); cudaFree(xz);
        check_cuda(e);
        if (err_h & DEVERR_TOO_MANY_VARS)
            throw std::runtime_error("Element valence exceeds maximum static valence passed to add_elements<..>(..)."
                                     " Please pass a large-enough static valence as template argument.");
        for (int64_t i = 0; i < n; ++i)
            for (int j = 0; j < vmax; ++j) counts[i] += rec_h[i * vmax + j] >= 0 ? 1 : 0;
        return counts;
    }
    template <int V, typename F>
    void add_group(std::map<int, std::vector<int32_t>>& groups, F& functor)
    {
        const auto it = groups.find(V);
        if (it != groups.end() && !it->second.empty()) add_elements<V>(it->second, functor);
    }

    SparseCSR pattern() const
    {
        int64_t nnz = 0;
        check(tad_hessian_nnz(p_, &nnz));
        SparseCSR H;
        H.rows = n_vars();
        H.outer.resize(n_vars() + 1);
        H.inner.resize(nnz);
        H.values.resize(nnz);
        check(tad_hessian_pattern(p_, H.outer.data(), H.inner.data()));
        return H;
    }
    void swap(ScalarFunction& o)
    {
        std::swap(p_, o.p_);
        std::swap(n_handles_, o.n_handles_);
        std::swap(terms_, o.terms_);
        std::swap(handle_bufs_, o.handle_bufs_);
        std::swap(term_sizes_, o.term_sizes_);
    }

    tad_problem* p_ = nullptr;
    int64_t n_handles_ = 0;
    std::vector<std::unique_ptr<detail::TermBase>> terms_;
    std::vector<int32_t*> handle_bufs_;
    std::vector<int64_t> term_sizes_;
};

/* VectorFunction<d> (include/TinyAD/VectorFunction.hh): elements return
   tad::Vec<T, M>, M residuals each, numbered term by term, element by
   element.  The inherited scalar methods act on the sum of squares |r|^2
   (eval_with_gradient: g = 2 J^T r; newton_solve: Gauss-Newton iterations
   with the Armijo line search on |r|^2). */
template <int d>
class VectorFunction : public ScalarFunction<d>
{
public:
    explicit VectorFunction(int64_t n_handles, const tad_settings* settings = nullptr) : ScalarFunction<d>(n_handles, settings) {}

    /* add_elements<N, M>(range, functor) (VectorFunction.hh:48-57) */
    template <int N, int M, typename Range, typename F>
    void add_elements(const Range& elements, F functor)
    {
        std::vector<int32_t> h;
        for (auto eh : elements) h.push_back((int32_t)eh);
        int32_t* hd = this->upload_handles(h);
        auto term = std::make_unique<detail::VecTerm<d, N, M, F>>(detail::HandleMapped<F>{functor, hd});
        check(tad_add_vector_elements_custom(this->p_, N, M, (int64_t)h.size(), &detail::term_callback, term.get()));
        this->terms_.push_back(std::move(term));
        this->term_sizes_.push_back((int64_t)h.size());
    }

    int64_t n_outputs() const { return tad_n_outputs(this->p_); }

    /* eval(x): the residual vector */
    std::vector<double> eval(const std::vector<double>& x) const
    {
        std::vector<double> r(n_outputs());
        check(tad_vec_eval(this->p_, x.data(), r.data()));
        return r;
    }
    std::vector<double> operator()(const std::vector<double>& x) const { return eval(x); }
    double eval_sum_of_squares(const std::vector<double>& x) const { return ScalarFunction<d>::eval(x); }

    std::tuple<std::vector<double>, SparseCSR> eval_with_jacobian(const std::vector<double>& x) const
    {
        std::vector<double> r(n_outputs());
        SparseCSR J = jacobian_pattern();
        check(tad_vec_eval_with_jacobian(this->p_, x.data(), r.data(), J.values.data()));
        return {std::move(r), std::move(J)};
    }

    /* (r, J, H): H[i] the Hessian of residual i (n_vars x n_vars, CSR) */
    std::tuple<std::vector<double>, SparseCSR, std::vector<SparseCSR>> eval_with_derivatives(const std::vector<double>& x) const
    {
        const int64_t m = n_outputs();
        std::vector<double> r(m);
        SparseCSR J = jacobian_pattern();
        int64_t nnz = 0;
        check(tad_vec_hessians_nnz(this->p_, &nnz));
        std::vector<int64_t> hp(m + 1);
        std::vector<int32_t> hr(nnz), hc(nnz);
        std::vector<double> hv(nnz);
        check(tad_vec_eval_with_derivatives(this->p_, x.data(), r.data(), J.values.data(), hp.data(), hr.data(), hc.data(),
                                            hv.data()));
        std::vector<SparseCSR> H(m);
        const int64_t n = this->n_vars();
        for (int64_t i = 0; i < m; ++i)
        {
            SparseCSR& Hi = H[i];
            Hi.rows = n;
            Hi.outer.assign(n + 1, 0);
            std::vector<std::tuple<int32_t, int32_t, double>> t;
            for (int64_t q = hp[i]; q < hp[i + 1]; ++q) t.emplace_back(hr[q], hc[q], hv[q]);
            std::sort(t.begin(), t.end());
            for (const auto& e : t)
            {
                ++Hi.outer[std::get<0>(e) + 1];
                Hi.inner.push_back(std::get<1>(e));
                Hi.values.push_back(std::get<2>(e));
            }
            for (int64_t r2 = 0; r2 < n; ++r2) Hi.outer[r2 + 1] += Hi.outer[r2];
        }
        return {std::move(r), std::move(J), std::move(H)};
    }

    /* (f, g, r, J), f = |r|^2, g = 2 J^T r (VectorFunctionImpl.hh:271-283) */
    std::tuple<double, std::vector<double>, std::vector<double>, SparseCSR>
    eval_sum_of_squares_with_derivatives(const std::vector<double>& x) const
    {
        double f;
        std::vector<double> g(this->n_vars()), r(n_outputs());
        SparseCSR J = jacobian_pattern();
        check(tad_eval_sum_of_squares_with_derivatives(this->p_, x.data(), &f, g.data(), r.data(), J.values.data()));
        return {f, std::move(g), std::move(r), std::move(J)};
    }

    /* gauss_newton_direction(r, J, solver, w) at x (GaussNewtonDirection.hh:24-47) */
    std::vector<double> gauss_newton_direction(const std::vector<double>& x, double w_identity = 0.0) const
    {
        std::vector<double> dvec(this->n_vars());
        const tad_status s = tad_gauss_newton_direction(this->p_, x.data(), w_identity, dvec.data(), nullptr, nullptr);
        if (s != TAD_OK && s != TAD_ERR_PCG_NOCONV) check(s);
        return dvec;
    }

private:
    SparseCSR jacobian_pattern() const
    {
        int64_t nnz = 0;
        check(tad_vec_jacobian_nnz(this->p_, &nnz));
        SparseCSR J;
        J.rows = n_outputs();
        J.cols = this->n_vars();
        J.outer.resize(J.rows + 1);
        J.inner.resize(nnz);
        J.values.resize(nnz);
        check(tad_vec_jacobian_pattern(this->p_, J.outer.data(), J.inner.data()));
        return J;
    }
};

/* vector_function<d>(range) (VectorFunction.hh:198-206) */
template <int d, typename Range>
VectorFunction<d> vector_function(const Range& variables, const tad_settings* settings = nullptr)
{
    int64_t n = 0;
    for (auto v : variables) { (void)v; ++n; }
    return VectorFunction<d>(n, settings);
}

/* scalar_function<d>(range) (ScalarFunctionImpl.hh:418-442) */
template <int d, typename Range>
ScalarFunction<d> scalar_function(const Range& variables, const tad_settings* settings = nullptr)
{
    int64_t n = 0;
    for (auto v : variables) { (void)v; ++n; }
    return ScalarFunction<d>(n, settings);
}

} // namespace tad
