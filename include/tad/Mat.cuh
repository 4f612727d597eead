/*
 * tad/Mat.cuh -- fixed-size vectors and matrices for element functors.
 *
 * Device code cannot use Eigen, so element functors use these instead of the
 * Eigen::Vector / Eigen::Matrix types of the reference's lambdas.  They are
 * generic over the entry type (passive double/float or tad::Scalar) and cover
 * what the reference's energies need: +, -, products, squaredNorm, dot,
 * determinant and inverse of 2x2 / 3x3 (adjugate over determinant), and
 * col_mat (include/TinyAD/Utils/Helpers.hh:48-76).  Storage is column-major.
 */
#pragma once
#include "Scalar.cuh"

namespace tad {

template <typename T, int R, int C = 1>
struct Mat
{
    T m[R * C];
    TAD_HD T& operator()(int i, int j) { return m[j * R + i]; }
    TAD_HD const T& operator()(int i, int j) const { return m[j * R + i]; }
    TAD_HD T& operator[](int i) { return m[i]; }
    TAD_HD const T& operator[](int i) const { return m[i]; }
    static constexpr int rows = R, cols = C;

    TAD_HD static Mat zero()
    {
        Mat r;
#pragma unroll
        for (int i = 0; i < R * C; ++i) r.m[i] = T(0);
        return r;
    }
    TAD_HD Mat<T, C, R> transpose() const
    {
        Mat<T, C, R> r;
#pragma unroll
        for (int i = 0; i < R; ++i)
#pragma unroll
            for (int j = 0; j < C; ++j) r(j, i) = (*this)(i, j);
        return r;
    }
    TAD_HD T squaredNorm() const
    {
        T acc = m[0] * m[0];
#pragma unroll
        for (int i = 1; i < R * C; ++i) acc = acc + m[i] * m[i];
        return acc;
    }
    TAD_HD T sum() const
    {
        T acc = m[0];
#pragma unroll
        for (int i = 1; i < R * C; ++i) acc = acc + m[i];
        return acc;
    }
};

template <typename T, int N> using Vec = Mat<T, N, 1>;

template <typename A, typename B>
using prod_t = decltype(std::declval<A>() * std::declval<B>());

template <typename A, typename B, int R, int C>
TAD_HD Mat<prod_t<A, B>, R, C> operator+(const Mat<A, R, C>& a, const Mat<B, R, C>& b)
{
    Mat<prod_t<A, B>, R, C> r;
#pragma unroll
    for (int i = 0; i < R * C; ++i) r.m[i] = a.m[i] + b.m[i];
    return r;
}
template <typename A, typename B, int R, int C>
TAD_HD Mat<prod_t<A, B>, R, C> operator-(const Mat<A, R, C>& a, const Mat<B, R, C>& b)
{
    Mat<prod_t<A, B>, R, C> r;
#pragma unroll
    for (int i = 0; i < R * C; ++i) r.m[i] = a.m[i] - b.m[i];
    return r;
}
template <typename A, int R, int C>
TAD_HD Mat<A, R, C> operator-(const Mat<A, R, C>& a)
{
    Mat<A, R, C> r;
#pragma unroll
    for (int i = 0; i < R * C; ++i) r.m[i] = -a.m[i];
    return r;
}
/* matrix product, summed over the inner index in order */
template <typename A, typename B, int R, int K, int C>
TAD_HD Mat<prod_t<A, B>, R, C> operator*(const Mat<A, R, K>& a, const Mat<B, K, C>& b)
{
    Mat<prod_t<A, B>, R, C> r;
#pragma unroll
    for (int j = 0; j < C; ++j)
#pragma unroll
        for (int i = 0; i < R; ++i)
        {
            prod_t<A, B> acc = a(i, 0) * b(0, j);
#pragma unroll
            for (int k = 1; k < K; ++k) acc = acc + a(i, k) * b(k, j);
            r(i, j) = acc;
        }
    return r;
}
/* scalar * matrix */
template <typename A, typename S, int R, int C, typename = std::enable_if_t<std::is_arithmetic<S>::value || is_scalar<S>::value>>
TAD_HD Mat<prod_t<A, S>, R, C> operator*(const Mat<A, R, C>& a, const S& s)
{
    Mat<prod_t<A, S>, R, C> r;
#pragma unroll
    for (int i = 0; i < R * C; ++i) r.m[i] = a.m[i] * s;
    return r;
}
template <typename A, typename S, int R, int C, typename = std::enable_if_t<std::is_arithmetic<S>::value || is_scalar<S>::value>>
TAD_HD Mat<prod_t<A, S>, R, C> operator*(const S& s, const Mat<A, R, C>& a) { return a * s; }

template <typename A, typename B, int N>
TAD_HD prod_t<A, B> dot(const Vec<A, N>& a, const Vec<B, N>& b)
{
    prod_t<A, B> acc = a[0] * b[0];
#pragma unroll
    for (int i = 1; i < N; ++i) acc = acc + a[i] * b[i];
    return acc;
}

template <typename T> TAD_HD T determinant(const Mat<T, 2, 2>& M) { return M(0, 0) * M(1, 1) - M(1, 0) * M(0, 1); }
template <typename T>
TAD_HD T determinant(const Mat<T, 3, 3>& M)
{
    return M(0, 0) * (M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2))
         - M(1, 0) * (M(0, 1) * M(2, 2) - M(2, 1) * M(0, 2))
         + M(2, 0) * (M(0, 1) * M(1, 2) - M(1, 1) * M(0, 2));
}

/* inverse = adjugate / determinant */
template <typename T>
TAD_HD Mat<T, 2, 2> inverse(const Mat<T, 2, 2>& M)
{
    const T id = T(1.0) / determinant(M);
    Mat<T, 2, 2> r;
    r(0, 0) = M(1, 1) * id;
    r(1, 0) = -M(1, 0) * id;
    r(0, 1) = -M(0, 1) * id;
    r(1, 1) = M(0, 0) * id;
    return r;
}
template <typename T>
TAD_HD Mat<T, 3, 3> inverse(const Mat<T, 3, 3>& M)
{
    Mat<T, 3, 3> c;   // cofactors
    c(0, 0) = M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2);
    c(0, 1) = M(2, 0) * M(1, 2) - M(1, 0) * M(2, 2);
    c(0, 2) = M(1, 0) * M(2, 1) - M(2, 0) * M(1, 1);
    c(1, 0) = M(2, 1) * M(0, 2) - M(0, 1) * M(2, 2);
    c(1, 1) = M(0, 0) * M(2, 2) - M(2, 0) * M(0, 2);
    c(1, 2) = M(2, 0) * M(0, 1) - M(0, 0) * M(2, 1);
    c(2, 0) = M(0, 1) * M(1, 2) - M(1, 1) * M(0, 2);
    c(2, 1) = M(1, 0) * M(0, 2) - M(0, 0) * M(1, 2);
    c(2, 2) = M(0, 0) * M(1, 1) - M(1, 0) * M(0, 1);
    const T det = M(0, 0) * c(0, 0) + M(1, 0) * c(1, 0) + M(2, 0) * c(2, 0);
    const T id = T(1.0) / det;
    Mat<T, 3, 3> r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) r(i, j) = c(j, i) * id;
    return r;
}

template <typename T, int R>
TAD_HD Mat<T, R, 2> col_mat(const Vec<T, R>& a, const Vec<T, R>& b)
{
    Mat<T, R, 2> M;
#pragma unroll
    for (int i = 0; i < R; ++i) { M(i, 0) = a[i]; M(i, 1) = b[i]; }
    return M;
}
template <typename T, int R>
TAD_HD Mat<T, R, 3> col_mat(const Vec<T, R>& a, const Vec<T, R>& b, const Vec<T, R>& c)
{
    Mat<T, R, 3> M;
#pragma unroll
    for (int i = 0; i < R; ++i) { M(i, 0) = a[i]; M(i, 1) = b[i]; M(i, 2) = c[i]; }
    return M;
}

} // namespace tad
