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

/* One Jacobi rotation in the (p, q) plane with precomputed (t, c): A <- J^T A J
   on the packed matrix, V <- V J */
template <int k, typename T>
TAD_HD void jacobi_rotate(T* A, T* V, int p, int q, T t, T c)
{
    const T s = t * c;
    const T apq = A[packed_index(p, q, k)];
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
    A[packed_index(p, p, k)] -= t * apq;
    A[packed_index(q, q, k)] += t * apq;
    A[packed_index(p, q, k)] = T(0);
#pragma unroll
    for (int r = 0; r < k; ++r)
    {
        const T vp = V[r * k + p], vq = V[r * k + q];
        V[r * k + p] = c * vp - s * vq;
        V[r * k + q] = s * vp + c * vq;
    }
}

/* In place: A packed (k(k+1)/2) -> eigenvalues on the diagonal, V (k*k,
   column l = eigenvector l, row-major V[r*k + l]).  Cyclic Jacobi in the
   round-robin (parallel) ordering: with n = k rounded up to even, a sweep is
   n - 1 rounds of n/2 disjoint pairs (the circle method: index n - 1 meets
   r, and (r + j, r - j) mod (n - 1) for j = 1 .. n/2 - 1; a pair with the
   padding index k of an odd k is skipped), so every pair is visited once per
   sweep.  The rotations of a round act on disjoint index pairs and commute:
   their angles are all taken from the matrix at the start of the round and
   are independent of one another, which a sweep in row order would chain
   (Golub & Van Loan 8.5.5 on the parallel orderings and their convergence). */
template <int k, typename T>
TAD_HD void jacobi_eigen_packed(T* A, T* V)
{
    constexpr int n = k + (k & 1), m = n - 1, np = n / 2;
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
        for (int r = 0; r < m; ++r)
        {
            int P[np], Q[np];
            T tt[np], cc[np];
#pragma unroll
            for (int j = 0; j < np; ++j)
            {
                const int a = j == 0 ? n - 1 : (r + j) % m, b = j == 0 ? r : (r + m - j) % m;
                P[j] = a < b ? a : b;
                Q[j] = a < b ? b : a;
            }
#pragma unroll
            for (int j = 0; j < np; ++j)
            {
                tt[j] = T(0);
                cc[j] = T(1);
                if (Q[j] >= k) continue;   // the padding index
                const T apq = A[packed_index(P[j], Q[j], k)];
                // FP32: no branch -- the fast angle maps a_pq = 0 to the identity rotation
                if (sizeof(T) == 8 && apq == T(0)) continue;
                jacobi_angle(A[packed_index(P[j], P[j], k)], A[packed_index(Q[j], Q[j], k)], apq, tt[j], cc[j]);
            }
#pragma unroll
            for (int j = 0; j < np; ++j)
                if (Q[j] < k && !(sizeof(T) == 8 && A[packed_index(P[j], Q[j], k)] == T(0)))
                    jacobi_rotate<k, T>(A, V, P[j], Q[j], tt[j], cc[j]);
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

/* ------------------------------------------------------------------------ */
/* Translation-deflated projection of an element Hessian                     */
/* ------------------------------------------------------------------------ */

/* 1 / sqrt((m+1)(m+2)), m = 0..7, as literals so that unrolled loops fold
   them to constants */
TAD_HD constexpr double helmert_scale(int m)
{
    return m == 0 ? 0.7071067811865475 : m == 1 ? 0.4082482904638631 : m == 2 ? 0.2886751345948129
         : m == 3 ? 0.22360679774997896 : m == 4 ? 0.18257418583505536 : m == 5 ? 0.1543033499620919
         : m == 6 ? 0.1336306209562122 : 0.11785113019775793;
}

/* Helmert basis of the complement of (1, ..., 1) in R^N (N <= 9): column m
   (0 <= m < N-1) is (1, ..., 1, -(m+1), 0, ...) / sqrt((m+1)(m+2)) with m+1
   leading ones.  Orthonormal, and orthogonal to the constant vector. */
TAD_HD constexpr double helmert(int a, int m)
{
    return a <= m ? helmert_scale(m) : (a == m + 1 ? -(m + 1.0) * helmert_scale(m) : 0.0);
}

/* Row-sum tolerance (relative to max |H_ij|) below which an element Hessian
   counts as translation invariant: a few hundred rounding units of the
   evaluation precision (4-byte types: FP32, else FP64). */
template <typename T> struct TranslationTol
{
    static constexpr double value = 256.0 * (sizeof(T) == 4 ? 1.1920928955078125e-07 : 2.220446049250313e-16);
};

/* Projection of the packed Hessian hp of an element with N vertices of d
   coordinates (variable a*d+p = coordinate p of vertex a), with the result of
   project_positive_definite<d*N>, for element energies that are invariant
   under translations of all N vertices (every energy of edge vectors or
   vertex differences: distortion, elasticity, Laplacian).
   For those the d translations t_p (t_p[a*d+p] = 1/sqrt(N)) are exact null
   vectors of H, hence eigenvectors with eigenvalue 0 (clamped to eps), and
   the other eigenpairs are those of the (d(N-1))^2 matrix A = Q^T H Q, Q =
   (Helmert basis of the complement of 1) x I_d.  The eigenproblem shrinks
   from k = dN to d(N-1) (k = 6 -> 4, 12 -> 9; the Jacobi cost goes with the
   cube).  The result is written in correction form,
       H + sum_{l: lambda_l(A) < eps} (eps - lambda_l) (Q v_l)(Q v_l)^T + eps sum_p t_p t_p^T,
   (for eps < 0, negative lambda_l flip: (|lambda_l| - lambda_l); the
   translations are left as they are), equal to V max(Lambda, eps) V^T in exact
   arithmetic.
   The diagonal-dominance early out of the general rule comes first (for
   eps < 0 its margin is negative and it can hold for invariant matrices).
   Returns 0 (hp unchanged) when it holds; -1 without touching hp when H is
   not translation invariant (some row sum H t_p above TranslationTol times
   max |H_ij|, or a non-finite entry): the caller then runs
   project_positive_definite<d*N>.  Otherwise returns 1 (hp projected). */
template <int d, int N, typename T, bool KnownInvariant = false>
TAD_HD int project_translation_deflated(T* hp, T eps)
{
    constexpr int k = d * N, R = d * (N - 1), NR = R * (R + 1) / 2;
    auto H = [&](int i, int j) -> T { return i <= j ? hp[packed_index(i, j, k)] : hp[packed_index(j, i, k)]; };
    // KnownInvariant: hp was built invariant (lift_translation_invariant of
    // an energy that declares it), so the row-sum test is skipped; its
    // diagonal then equals minus the off-diagonal sum of its coordinate, and
    // the dominance early out can only hold for eps <= 0
    if (!KnownInvariant || !(eps > T(0)))
        if (positive_diagonally_dominant<k, T>(hp, eps)) return 0;
    if constexpr (!KnownInvariant)
    {
        T hmax = T(0);
#pragma unroll
        for (int q = 0; q < k * (k + 1) / 2; ++q) hmax = tad_abs(hp[q]) > hmax ? tad_abs(hp[q]) : hmax;
        T rmax = T(0);
#pragma unroll
        for (int i = 0; i < k; ++i)
#pragma unroll
            for (int q = 0; q < d; ++q)
            {
                T s = T(0);
#pragma unroll
                for (int b = 0; b < N; ++b) s += H(i, b * d + q);
                rmax = tad_abs(s) > rmax ? tad_abs(s) : rmax;
            }
        if (!(rmax <= T(TranslationTol<T>::value) * hmax) || !(hmax < T(INFINITY))) return -1;
    }
    // A = Q^T (H Q) (packed R x R, reduced index m*d + p), streamed over the
    // rows i = a*d + p of H: w = (H Q)[i][J] is formed and at once added to
    // the rows (m, p) of A with Q[a][m] != 0 (m >= a-1), so no k x R
    // intermediate is held
    T A[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) A[q] = T(0);
#pragma unroll
    for (int i = 0; i < k; ++i)
    {
        const int a = i / d, p = i % d;
#pragma unroll
        for (int J = 0; J < R; ++J)
        {
            const int m2 = J / d, q = J % d;
            if ((a > 0 ? a - 1 : 0) * d + p > J) continue;   // no (m, p) <= J receives this entry
            T w = T(0);
#pragma unroll
            for (int b = 0; b <= m2 + 1; ++b) w += H(i, b * d + q) * T(helmert(b, m2));
#pragma unroll
            for (int m = (a > 0 ? a - 1 : 0); m < N - 1; ++m)
                if (m * d + p <= J) A[packed_index(m * d + p, J, R)] += T(helmert(a, m)) * w;
        }
    }
    T V[R * R];
    T lam0[R];
    jacobi_eigen_packed<R, T>(A, V);
#pragma unroll
    for (int l = 0; l < R; ++l)
    {
        const T lv = A[packed_index(l, l, R)];
        T c = T(0);
        if (eps < T(0)) { if (lv < T(0)) c = -lv - lv; }
        else if (lv < eps) c = eps - lv;
        lam0[l] = c;
    }
    // clamped modes, lifted back: w = Q v_l
#pragma unroll
    for (int l = 0; l < R; ++l)
    {
        if (lam0[l] == T(0)) continue;
        T w[k];
#pragma unroll
        for (int a = 0; a < N; ++a)
#pragma unroll
            for (int p = 0; p < d; ++p)
            {
                T s = T(0);
#pragma unroll
                for (int m = (a > 0 ? a - 1 : 0); m < N - 1; ++m) s += T(helmert(a, m)) * V[(m * d + p) * R + l];
                w[a * d + p] = s;
            }
#pragma unroll
        for (int i = 0; i < k; ++i)
#pragma unroll
            for (int j = i; j < k; ++j) hp[packed_index(i, j, k)] += lam0[l] * w[i] * w[j];
    }
    if (eps > T(0))
    {
        const T c = eps / T(N);
#pragma unroll
        for (int a = 0; a < N; ++a)
#pragma unroll
            for (int b = 0; b < N; ++b)
#pragma unroll
                for (int p = 0; p < d; ++p)
                    if (a * d + p <= b * d + p) hp[packed_index(a * d + p, b * d + p, k)] += c;
    }
    return 1;
}

/* Element projection: the translation-deflated form where it applies (N >= 2
   and H translation invariant), else the general one.  Returns true if hp was
   changed. */
template <int d, int N, typename T>
TAD_HD bool project_element_hessian(T* hp, T eps)
{
    if constexpr (N >= 2 && N <= 9)
    {
        const int r = project_translation_deflated<d, N, T>(hp, eps);
        if (r >= 0) return r > 0;
    }
    return project_positive_definite<d * N, T>(hp, eps);
}

} // namespace tad
