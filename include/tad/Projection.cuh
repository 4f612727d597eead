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
 * FP32 (mixed-precision mode only): the same clamp at eps, but step 3 adds
 * only the corrections of the clamped modes,
 *   H + sum_{i: lambda_i < eps} (eps - lambda_i) v_i v_i^T,
 * which equals the rebuilt V max(Lambda, eps) V^T in exact arithmetic.  A
 * full FP32 rebuild rounds every entry of the block (~k eps_fp32
 * max|lambda|), including the unclamped part; the correction form leaves
 * that part as evaluated.  The clamp level must stay at eps: raising it to
 * the FP32 resolution of the spectrum (a floor ~ k eps_fp32 max|lambda|)
 * adds a stiffness to every element's near-null (rigid) modes that, summed
 * over a large mesh, swamps the smallest eigenvalues of the assembled
 * Hessian and turns Newton's convergence linear (measured: 55 instead of 25
 * iterations to 1e-8 energy error on a 1.64M-face disk parametrisation).
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

/* Rotation (c, s = t c) that zeroes a_pq (Golub & Van Loan, 8.5.2):
   theta = (a_qq - a_pp) / (2 a_pq), t = sign(theta) / (|theta| + sqrt(theta^2 + 1)),
   c = 1 / sqrt(t^2 + 1).  Only c^2 + s^2 = 1 matters for the result (it keeps
   the transformation orthogonal); t itself only decides how well a_pq is
   zeroed, which the next sweep corrects.  FP32 on the device therefore takes
   theta and t from the fast divide / reciprocal square root and refines c
   with one Newton step for 1/sqrt (y <- y (3 - x y^2) / 2), which brings
   c^2 (1 + t^2) to within a few ulp of 1. */
template <typename T>
TAD_HD void jacobi_angle(T app, T aqq, T apq, T& t, T& c)
{
    if (apq == T(0)) { t = T(0); c = T(1); return; }
    const T theta = (aqq - app) / (T(2) * apq);
    t = (theta >= T(0) ? T(1) : T(-1)) / (tad_abs(theta) + tad_sqrt(theta * theta + T(1)));
    c = T(1) / tad_sqrt(t * t + T(1));
}
#if defined(__CUDA_ARCH__)
template <>
__device__ __forceinline__ void jacobi_angle<float>(float app, float aqq, float apq, float& t, float& c)
{
    const float theta = __fdividef(aqq - app, 2.0f * apq);
    const float h = fmaf(theta, theta, 1.0f);
    const float sq = h * rsqrtf(h);                            // sqrt(theta^2 + 1), approximate
    t = copysignf(__fdividef(1.0f, fabsf(theta) + sq), theta);
    if (!(h < 3.0e38f)) t = 0.0f;                              // |theta| beyond FP32 range: no rotation needed
    const float u = fmaf(t, t, 1.0f);
    float y = rsqrtf(u);
    y = y * fmaf(-0.5f * u, y * y, 1.5f);                      // Newton step for 1/sqrt(u)
    c = y;
}
#endif

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
                // FP32: no branch -- the fast angle maps a_pq = 0 to the identity rotation
                if (sizeof(T) == 8 && apq == T(0)) continue;
                const T app = A[packed_index(p, p, k)], aqq = A[packed_index(q, q, k)];
                T t, c;
                jacobi_angle(app, aqq, apq, t, c);
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
#pragma unroll
    for (int i = 0; i < k; ++i)
    {
        T l = A[packed_index(i, i, k)];
        if (eps < T(0)) { if (l < T(0)) { l = -l; all_positive = false; } }
        else if (l < eps) { l = eps; all_positive = false; }
        lam[i] = l;
    }
    if (all_positive) return false;
    if (sizeof(T) == 4)
    {
        // correction form: only the clamped modes change
#pragma unroll
        for (int i = 0; i < k; ++i) lam[i] -= A[packed_index(i, i, k)];
#pragma unroll
        for (int i = 0; i < k; ++i)
#pragma unroll
            for (int j = i; j < k; ++j)
            {
                T acc = hp[packed_index(i, j, k)];
#pragma unroll
                for (int l = 0; l < k; ++l) acc += V[i * k + l] * lam[l] * V[j * k + l];
                hp[packed_index(i, j, k)] = acc;
            }
        return true;
    }
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
