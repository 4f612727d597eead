/*
 * tad/Energies.cuh -- the library's built-in element functors (tad_energy in
 * tad.h).  They are ordinary element functors, written like the reference's
 * test lambdas, and run through the same kernels as user functors.
 *
 *   SymmetricDirichletTri  tests/NewtonTest.cc:28-44 (weight per element)
 *   SymmetricDirichletTet  its 3D analogue (k = 12)
 *   PositionPenalty        tests/NewtonTest.cc:48-55 (weight per element)
 *   Quadratic              the quadratics of tests/ScalarFunctionTest.cc
 *   DirichletTri           the Laplacian energy of tests/DynamicElementsTest.cc:60-91
 * and the residual functors of vector terms (VectorFunction):
 *   SymmetricDirichletTriResiduals  the 8 residuals of tests/GaussNewtonTest.cc:33-66
 *   PositionResiduals      the 2 residuals of tests/GaussNewtonTest.cc:67-74
 *
 * Each functor reads its element's vertex handles (`vtx`, n_elem x N) and
 * parameters (`prm`, n_elem x P) through element.handle, the way the
 * reference lambdas read F(element.handle, i).
 */
#pragma once
#include <math.h>
#include <stdint.h>
#include "Mat.cuh"
#include "Element.cuh"

namespace tad {

struct SymmetricDirichletTri
{
    static constexpr int d = 2, N = 3, n_params = 5;
    static constexpr bool translation_invariant = true;   // a function of edge vectors
    const int32_t* vtx;
    const double* prm;

    template <typename El>
    TAD_HD auto operator()(El& element) const -> TAD_SCALAR_TYPE(element)
    {
        using T = TAD_SCALAR_TYPE(element);
        using P = TAD_PASSIVE_TYPE(element);
        const int64_t e = element.handle;
        const double* p = prm + e * n_params;
        Mat<P, 2, 2> Mr;
#pragma unroll
        for (int i = 0; i < 4; ++i) Mr.m[i] = P(p[i]);
        const Vec<T, 2> a = element.variables(vtx[e * 3 + 0]);
        const Vec<T, 2> b = element.variables(vtx[e * 3 + 1]);
        const Vec<T, 2> c = element.variables(vtx[e * 3 + 2]);
        const Mat<T, 2, 2> M = col_mat(b - a, c - a);
        if (determinant(M) <= 0.0) return T(INFINITY);
        return ((M * inverse(Mr)).squaredNorm() + (Mr * inverse(M)).squaredNorm()) * P(p[4]);
    }
};

struct SymmetricDirichletTet
{
    static constexpr int d = 3, N = 4, n_params = 10;
    static constexpr bool translation_invariant = true;   // a function of edge vectors
    const int32_t* vtx;
    const double* prm;

    template <typename El>
    TAD_HD auto operator()(El& element) const -> TAD_SCALAR_TYPE(element)
    {
        using T = TAD_SCALAR_TYPE(element);
        using P = TAD_PASSIVE_TYPE(element);
        const int64_t e = element.handle;
        const double* p = prm + e * n_params;
        Mat<P, 3, 3> Mr;
#pragma unroll
        for (int i = 0; i < 9; ++i) Mr.m[i] = P(p[i]);
        const Vec<T, 3> a = element.variables(vtx[e * 4 + 0]);
        const Vec<T, 3> b = element.variables(vtx[e * 4 + 1]);
        const Vec<T, 3> c = element.variables(vtx[e * 4 + 2]);
        const Vec<T, 3> dd = element.variables(vtx[e * 4 + 3]);
        const Mat<T, 3, 3> M = col_mat(b - a, c - a, dd - a);
        if (determinant(M) <= 0.0) return T(INFINITY);
        return ((M * inverse(Mr)).squaredNorm() + (Mr * inverse(M)).squaredNorm()) * P(p[9]);
    }
};

template <int D>
struct PositionPenalty
{
    static constexpr int d = D, N = 1, n_params = D + 1;
    const int32_t* vtx;
    const double* prm;

    template <typename El>
    TAD_HD auto operator()(El& element) const -> TAD_SCALAR_TYPE(element)
    {
        using T = TAD_SCALAR_TYPE(element);
        using P = TAD_PASSIVE_TYPE(element);
        const int64_t e = element.handle;
        const double* p = prm + e * n_params;
        Vec<P, D> target;
#pragma unroll
        for (int i = 0; i < D; ++i) target[i] = P(p[i]);
        const Vec<T, D> x = element.variables(vtx[e]);
        return (target - x).squaredNorm() * P(p[D]);
    }
};

/* E = sum_ij A_ij x_i x_j + sum_i b_i x_i + c over the element's variables */
template <int D, int NV>
struct Quadratic
{
    static constexpr int d = D, N = NV, k = D * NV, n_params = D * NV * D * NV + D * NV + 1;
    const int32_t* vtx;
    const double* prm;

    template <typename El>
    TAD_HD auto operator()(El& element) const -> TAD_SCALAR_TYPE(element)
    {
        using T = TAD_SCALAR_TYPE(element);
        using P = TAD_PASSIVE_TYPE(element);
        const int64_t e = element.handle;
        const double* p = prm + e * n_params;
        T xs[k];
#pragma unroll
        for (int n = 0; n < NV; ++n)
        {
            const Vec<T, D> v = element.variables(vtx[e * NV + n]);
#pragma unroll
            for (int i = 0; i < D; ++i) xs[n * D + i] = v[i];
        }
        T acc = T(P(p[k * k + k]));
#pragma unroll
        for (int i = 0; i < k; ++i)
#pragma unroll
            for (int j = 0; j < k; ++j)
                if (p[i * k + j] != 0.0) acc = acc + P(p[i * k + j]) * xs[i] * xs[j];
#pragma unroll
        for (int i = 0; i < k; ++i)
            if (p[k * k + i] != 0.0) acc = acc + P(p[k * k + i]) * xs[i];
        return acc;
    }
};

template <int D>
struct DirichletTri
{
    static constexpr int d = D, N = 3, n_params = 1;
    static constexpr bool translation_invariant = true;   // a function of edge vectors
    const int32_t* vtx;
    const double* prm;

    template <typename El>
    TAD_HD auto operator()(El& element) const -> TAD_SCALAR_TYPE(element)
    {
        using T = TAD_SCALAR_TYPE(element);
        using P = TAD_PASSIVE_TYPE(element);
        const int64_t e = element.handle;
        const Vec<T, D> a = element.variables(vtx[e * 3 + 0]);
        const Vec<T, D> b = element.variables(vtx[e * 3 + 1]);
        const Vec<T, D> c = element.variables(vtx[e * 3 + 2]);
        return ((b - a).squaredNorm() + (c - b).squaredNorm() + (a - c).squaredNorm()) * P(prm[e]);
    }
};

} // namespace tad

namespace tad {

/* Symmetric Dirichlet of one triangle as a function of its UVs (a, b, c)
   and of its 3D rest positions (Pa, Pb, Pc): the rest edge matrix is the
   triangle in its own orthonormal frame, Mr = [[l, e.f/l], [0, |e x f|/l]]
   with e = Pb - Pa, f = Pc - Pa, l = |e|, and the weight is the rest area
   |e x f| / 2 -- the same formulas that produce the [Mr, w] parameters of
   SymmetricDirichletTri.  Used by the adjoint (mixed second derivatives
   d2E/dx dP); S is any scalar type (double, tad::MixedScalar, ...). */
template <typename S>
TAD_HD S symmetric_dirichlet_tri_rest(const Vec<S, 2>& a, const Vec<S, 2>& b, const Vec<S, 2>& c,
                                      const Vec<S, 3>& Pa, const Vec<S, 3>& Pb, const Vec<S, 3>& Pc)
{
    using std::sqrt;
    const Vec<S, 3> e = Pb - Pa;
    const Vec<S, 3> f = Pc - Pa;
    const S l = sqrt(dot(e, e));
    Vec<S, 3> n;
    n[0] = e[1] * f[2] - e[2] * f[1];
    n[1] = e[2] * f[0] - e[0] * f[2];
    n[2] = e[0] * f[1] - e[1] * f[0];
    const S an = sqrt(dot(n, n));
    Mat<S, 2, 2> Mr;
    Mr(0, 0) = l;
    Mr(1, 0) = S(0.0);
    Mr(0, 1) = dot(e, f) / l;
    Mr(1, 1) = an / l;
    const Mat<S, 2, 2> M = col_mat(b - a, c - a);
    if (to_passive(determinant(M)) <= 0.0) return S(INFINITY);
    return ((M * inverse(Mr)).squaredNorm() + (Mr * inverse(M)).squaredNorm()) * (an * 0.5);
}

/* Residual form of SymmetricDirichletTri: sqrt(w) times the entries of
   J = M Mr^-1 and of J^-1 = Mr M^-1 (row-major, J first), so the sum of
   squares is the symmetric Dirichlet energy (tests/GaussNewtonTest.cc:33-66,
   weight 1/#F there).  Params as SymmetricDirichletTri: Mr (column-major), w. */
struct SymmetricDirichletTriResiduals
{
    static constexpr int d = 2, N = 3, M = 8, n_params = 5;
    const int32_t* vtx;
    const double* prm;

    template <typename El>
    TAD_HD auto operator()(El& element) const -> Vec<TAD_SCALAR_TYPE(element), 8>
    {
        using T = TAD_SCALAR_TYPE(element);
        using P = TAD_PASSIVE_TYPE(element);
        const int64_t e = element.handle;
        const double* p = prm + e * n_params;
        Mat<P, 2, 2> Mr;
#pragma unroll
        for (int i = 0; i < 4; ++i) Mr.m[i] = P(p[i]);
        const Vec<T, 2> a = element.variables(vtx[e * 3 + 0]);
        const Vec<T, 2> b = element.variables(vtx[e * 3 + 1]);
        const Vec<T, 2> c = element.variables(vtx[e * 3 + 2]);
        const Mat<T, 2, 2> Mt = col_mat(b - a, c - a);
        Vec<T, 8> E;
        if (determinant(Mt) <= 0.0)
        {
#pragma unroll
            for (int o = 0; o < 8; ++o) E[o] = T(INFINITY);
            return E;
        }
        const Mat<T, 2, 2> J = Mt * inverse(Mr);
        const Mat<T, 2, 2> Ji = Mr * inverse(Mt);
        using std::sqrt;
        const P s = P(sqrt(p[4]));
        E[0] = J(0, 0) * s; E[1] = J(0, 1) * s; E[2] = J(1, 0) * s; E[3] = J(1, 1) * s;
        E[4] = Ji(0, 0) * s; E[5] = Ji(0, 1) * s; E[6] = Ji(1, 0) * s; E[7] = Ji(1, 1) * s;
        return E;
    }
};

/* Residual form of PositionPenalty: sqrt(w) (target - p), D residuals
   (tests/GaussNewtonTest.cc:67-74).  Params: target (D), w. */
template <int D>
struct PositionResiduals
{
    static constexpr int d = D, N = 1, M = D, n_params = D + 1;
    const int32_t* vtx;
    const double* prm;

    template <typename El>
    TAD_HD auto operator()(El& element) const -> Vec<TAD_SCALAR_TYPE(element), D>
    {
        using T = TAD_SCALAR_TYPE(element);
        using P = TAD_PASSIVE_TYPE(element);
        const int64_t e = element.handle;
        const double* p = prm + e * n_params;
        using std::sqrt;
        const P s = P(sqrt(p[D]));
        const Vec<T, D> x = element.variables(vtx[e]);
        Vec<T, D> r;
#pragma unroll
        for (int i = 0; i < D; ++i) r[i] = (P(p[i]) - x[i]) * s;
        return r;
    }
};

} // namespace tad
