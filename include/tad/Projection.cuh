/*
 * tad/Projection.cuh -- per-element PSD projection of a packed symmetric
 * k x k Hessian, with the rules of TinyAD's project_positive_definite
 * (include/TinyAD/Utils/HessianProjection.hh:16-101):
 *   1. early out if the matrix is diagonally dominant with positive
 *      diagonal by at least eps (sufficient for PD, Gershgorin);
 *   2. eigendecompose; clamp eigenvalues below eps to eps (or, if eps < 0,
 *      flip negative eigenvalues to their absolute value);
 *   3. if nothing was clamped leave H unchanged, else rebuild V D V^T.
 * The eigensolver is cyclic Jacobi (Golub & Van Loan, Matrix Computations,
 * 8.5) run in the element's own thread on registers / local memory; the
 * clamped spectral projector is unique, so the result matches any accurate
 * eigensolver (the reference uses Eigen's SelfAdjointEigenSolver) up to
 * rounding.
 *
 * FP32 (mixed-precision mode only): the clamp level is raised to
 * max(eps, 8 k eps_fp32 max|lambda|).  Rebuilding V D V^T in FP32 perturbs
 * the eigenvalues by up to ~k^2 eps_fp32 max|lambda|, so clamping to eps
 * alone can leave an indefinite element block, and an indefinite assembled
 * Hessian breaks conjugate gradients on problems whose Hessian has
 * near-null directions (rigid motions of an unconstrained parametrisation).
 * The floor is below the resolution of an FP32 eigendecomposition, so it
 * removes nothing FP32 could represent.
 */
#pragma once
#include "Scalar.cuh"

namespace tad {

template <int k, typename T>
TAD_HD bool positive_diagonally_dominant(const T* hp, T eps)
{
    bool dd = true;
#pragma unroll
    for (int i = 0; i < k; ++i)
    {
        T off = T(0);
#pragma unroll
        for (int j = 0; j < k; ++j)
            if (j != i) off += (j > i ? (hp[packed_index(i, j, k)] < T(0) ? -hp[packed_index(i, j, k)] : hp[packed_index(i, j, k)])
                                      : (hp[packed_index(j, i, k)] < T(0) ? -hp[packed_index(j, i, k)] : hp[packed_index(j, i, k)]));
        if (hp[packed_index(i, i, k)] < off + eps) dd = false;
    }
    return dd;
}

template <typename T> TAD_HD T tad_abs(T v) { return v < T(0) ? -v : v; }
template <typename T> TAD_HD T tad_sqrt(T v) { using std::sqrt; return sqrt(v); }

/* max Jacobi sweeps: quadratic convergence reaches rounding level in 5-7 */
template <typename T> struct JacobiSweeps { static constexpr int value = 10; };
template <> struct JacobiSweeps<float> { static constexpr int value = 8; };

/* In place: A packed (k(k+1)/2) -> eigenvalues on the diagonal, V (k*k,
   column l = eigenvector l, row-major V[r*k + l]) */
template <int k, typename T>
TAD_HD void jacobi_eigen_packed(T* A, T* V)
{
#pragma unroll
    for (int r = 0; r < k; ++r)
#pragma unroll
        for (int l = 0; l < k; ++l) V[r * k + l] = (r == l) ? T(1) : T(0);
    T fro = T(0);
#pragma unroll
    for (int q = 0; q < k * (k + 1) / 2; ++q) fro += A[q] * A[q];
    const T tol = (sizeof(T) == 8 ? T(1e-34) : T(1e-15)) * fro;   // (rel. off-norm)^2
#pragma unroll 1
    for (int sweep = 0; sweep < JacobiSweeps<T>::value; ++sweep)
    {
        T off = T(0);
#pragma unroll
        for (int p = 0; p < k; ++p)
#pragma unroll
            for (int q = p + 1; q < k; ++q) off += A[packed_index(p, q, k)] * A[packed_index(p, q, k)];
        if (!(off > tol)) break;
#pragma unroll
        for (int p = 0; p < k - 1; ++p)
#pragma unroll
            for (int q = p + 1; q < k; ++q)
            {
                const T apq = A[packed_index(p, q, k)];
                if (apq == T(0)) continue;
                const T app = A[packed_index(p, p, k)], aqq = A[packed_index(q, q, k)];
                const T theta = (aqq - app) / (T(2) * apq);
                const T t = (theta >= T(0) ? T(1) : T(-1)) / (tad_abs(theta) + tad_sqrt(theta * theta + T(1)));
                const T c = T(1) / tad_sqrt(t * t + T(1));
                const T s = t * c;
#pragma unroll
                for (int r = 0; r < k; ++r)
                {
                    if (r == p || r == q) continue;
                    const int ip = r < p ? packed_index(r, p, k) : packed_index(p, r, k);
                    const int iq = r < q ? packed_index(r, q, k) : packed_index(q, r, k);
                    const T arp = A[ip], arq = A[iq];
                    A[ip] = c * arp - s * arq;
                    A[iq] = s * arp + c * arq;
                }
                A[packed_index(p, p, k)] = app - t * apq;
                A[packed_index(q, q, k)] = aqq + t * apq;
                A[packed_index(p, q, k)] = T(0);
#pragma unroll
                for (int r = 0; r < k; ++r)
                {
                    const T vp = V[r * k + p], vq = V[r * k + q];
                    V[r * k + p] = c * vp - s * vq;
                    V[r * k + q] = s * vp + c * vq;
                }
            }
    }
}

template <typename T> struct ProjectionFloor { static constexpr double rel = 0.0; };
template <> struct ProjectionFloor<float> { static constexpr double rel = 8.0 * 1.1920928955078125e-07; };

/* Projects the packed symmetric k x k matrix hp in place.  Returns true if
   the matrix was changed. */
template <int k, typename T>
TAD_HD bool project_positive_definite(T* hp, T eps)
{
    if (k == 0) return false;
    if (positive_diagonally_dominant<k, T>(hp, eps)) return false;
    constexpr int NP = k * (k + 1) / 2;
    T A[NP];
    T V[k * k];
#pragma unroll
    for (int q = 0; q < NP; ++q) A[q] = hp[q];
    jacobi_eigen_packed<k, T>(A, V);
    T lam[k];
    bool all_positive = true;
    T floor_eps = eps;
    if (ProjectionFloor<T>::rel > 0.0 && eps >= T(0))
    {
        T amax = T(0);
#pragma unroll
        for (int i = 0; i < k; ++i) amax = tad_abs(A[packed_index(i, i, k)]) > amax ? tad_abs(A[packed_index(i, i, k)]) : amax;
        const T fl = T(ProjectionFloor<T>::rel * k) * amax;
        floor_eps = fl > eps ? fl : eps;
    }
#pragma unroll
    for (int i = 0; i < k; ++i)
    {
        T l = A[packed_index(i, i, k)];
        if (eps < T(0)) { if (l < T(0)) { l = -l; all_positive = false; } }
        else if (l < floor_eps) { l = floor_eps; all_positive = false; }
        lam[i] = l;
    }
    if (all_positive) return false;
#pragma unroll
    for (int i = 0; i < k; ++i)
#pragma unroll
        for (int j = i; j < k; ++j)
        {
            T acc = T(0);
#pragma unroll
            for (int l = 0; l < k; ++l) acc += V[i * k + l] * lam[l] * V[j * k + l];
            hp[packed_index(i, j, k)] = acc;
        }
    return true;
}

} // namespace tad
