/*
 * tad/ElementKernels.cuh -- element evaluation kernels, templated on the
 * variable dimension d, the valence N and the element functor.  Included by
 * the library for its built-in energies and by the C++ front end for user
 * functors, so both run the same code.
 *
 * One element per thread.  The functor runs with an element whose
 * variables() seed tad::Scalar<k> values (k = d*N) held in registers; the
 * result (value, gradient, packed Hessian) is optionally PSD-projected
 * (tad/Projection.cuh: translation-deflated where the element Hessian allows
 * it, else the general form in a second pass) and written as
 *   f:  double  out_f[e]
 *   g:  out_g[e][N*d] (slot-major): double, or -- in the mixed second-order
 *       modes (T = float, HESSIAN / HESSIAN_PROJ) -- a double-float pair
 *       (hi, lo floats, the same 8 bytes) that the mixed assembly sums
 *       without FP64 instructions
 *   H:  Th      out_H[e][N(N+1)/2 slot pairs a<=b][d][d]
 * which the assembly kernels gather per global block in element order.  This
 * replaces the per-element std::vector results and the serial triplet
 * scatter of ScalarObjectiveTerm::eval_with_derivatives_add
 * (include/TinyAD/Detail/ScalarObjectiveTerm.hh:224-278).
 */
#pragma once
#include <stdint.h>
#include <algorithm>
#include <type_traits>
#include "Scalar.cuh"
#include "Element.cuh"
#include "Projection.cuh"
#include "RowIO.cuh"
#include "../tad.h"

namespace tad {

template <typename T> __device__ __forceinline__ bool finite_val(T v) { return ::isfinite(v); }

struct ElemLaunch
{
    int64_t n_elem;
    const int32_t* rec;      /* recorded access order, n_elem * N, -1 = unused */
    const double* x;
    const double* dir;
    const double* steps;     /* device, n_steps */
    int n_steps;
    int64_t f_stride;        /* line search: row stride of out_f */
    double eps;
    int project;
    double* out_f;
    void* out_g;
    void* out_H;
    int32_t* record;         /* record mode output */
    int32_t* err;
    double* out_r;           /* vector terms: residuals [n_elem][M] */
    double* out_J;           /* vector terms: residual gradients [n_elem][M][k] */
    double* out_Hv;          /* vector terms: packed residual Hessians [n_elem][M][k(k+1)/2] */
    uint32_t* proj_list;     /* HESSIAN_PROJ: [0] count, [1..] elements left for the general projection */
    const int32_t* active;   /* NULL or a device int; 0 = nothing to do (line search, second order) */
};

template <int d, int N, typename Energy>
__global__ void __launch_bounds__(128) k_elem_value(ElemLaunch L, Energy energy)
{
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= L.n_elem) return;
    PassiveElement<d, N, double> el{e, L.x};
    L.out_f[e] = (double)energy(el);
}

/* f at x + s_j dir for the n_steps trial step sizes, evaluated in the passive
   type P (double; the double-float of mixed mode for k <= 8) */
template <int d, int N, typename Energy, typename P = double>
__global__ void __launch_bounds__(128) k_elem_linesearch(ElemLaunch L, Energy energy)
{
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= L.n_elem || (L.active && *L.active == 0)) return;
    for (int j = 0; j < L.n_steps; ++j)
    {
        LineSearchElement<d, N, P> el{e, L.x, L.dir, P(L.steps[j])};
        L.out_f[(int64_t)j * L.f_stride + e] = (double)energy(el);
    }
}

template <int d, int N, typename Energy>
__global__ void __launch_bounds__(128) k_elem_record(ElemLaunch L, Energy energy)
{
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= L.n_elem) return;
    RecordElement<d, N> el;
    el.handle = e;
    el.x = L.x;
#pragma unroll
    for (int i = 0; i < N; ++i) el.vh[i] = -1;
    (void)energy(el);
    if (el.overflow) report_error(L.err, DEVERR_TOO_MANY_VARS);
#pragma unroll
    for (int i = 0; i < N; ++i) L.record[e * N + i] = (i < el.n) ? el.vh[i] : -1;
}

template <int d, int N, typename Energy>
__global__ void __launch_bounds__(128) k_elem_gradient(ElemLaunch L, Energy energy)
{
    constexpr int k = d * N;
    using S = Scalar<k, double, false>;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= L.n_elem) return;
    ActiveElement<d, N, S> el;
    el.handle = e;
    el.x = L.x;
    el.err = L.err;
#pragma unroll
    for (int i = 0; i < N; ++i) el.vh[i] = L.rec[e * N + i];
    const S r = energy(el);
    L.out_f[e] = r.val;
    double* g = (double*)L.out_g + e * k;
    bool fin = true;
#pragma unroll
    for (int i = 0; i < k; ++i) { g[i] = r.grad[i]; fin = fin && finite_val(r.grad[i]); }
    if (!fin) report_error(L.err, DEVERR_NONFINITE);
}

/* value and gradient types of the second-order kernel: FP64 for the plain
   path; for the mixed path double-float (FP32-pipe arithmetic, ~48-bit
   significand) up to k = 8 and FP64 beyond.  The tetrahedron (k = 12, 9
   derivatives after the translation reduction) is bound by register spills
   of its Hessians, not by the FP64 pipe: with a double-float value and
   gradient it measured 8.33 instead of 6.60 ms on 663,552 tets. */
template <typename T, int K> struct ValOf { using type = double; };
template <int K> struct ValOf<float, K> { using type = std::conditional_t<(K <= 8), DoubleFloatValue, double>; };
template <typename T, int K> struct GradOf { using type = double; };
template <int K> struct GradOf<float, K> { using type = std::conditional_t<(K <= 8), DoubleFloat, double>; };

/* For k <= 8 the PSD projection runs in its own kernel (k_project_blocks)
   over the element blocks the evaluation kernel wrote, at 64 registers a
   thread against the evaluation's 128.  On the 1.64M-face disk (k = 6,
   reduced mixed evaluation, deflated 4 x 4 projection) the split pair takes
   0.394 ms; fused into the evaluation it takes 0.395 / 0.429 / 0.510 ms
   with launch bounds of 4 / 3 / 2 resident blocks per SM -- the
   projection's registers cost the evaluation spills or occupancy, which
   outweighs the block re-read.  At k = 12 the
   evaluation alone spills, and a second pass only adds traffic (13.6 ms
   fused, 18.4 ms split on 663,552 tets with the full 12 x 12 projection), so
   it stays fused. */
template <int k> struct FusedProjection { static constexpr bool value = k > 8; };

/* Valences whose elements try the translation-deflated projection
   (project_translation_deflated); elements that are not translation
   invariant are appended to L.proj_list and projected by
   k_project_general, which keeps the general k x k eigensolver (and its
   registers) out of the evaluation and block-projection kernels. */
template <int N> struct DeflatedProjection { static constexpr bool value = N >= 2 && N <= 9; };

__device__ __forceinline__ void defer_projection(const ElemLaunch& L, int64_t e)
{
    if (!L.proj_list) { report_error(L.err, DEVERR_NO_PROJ_LIST); return; }
    const uint32_t slot = atomicAdd(L.proj_list, 1u);
    L.proj_list[1 + slot] = (uint32_t)e;
}

/* PSD projection of an element Hessian in an element kernel: the deflated
   form where the valence allows it, with non-invariant elements deferred */
template <int d, int N, typename T, bool KnownInvariant = false>
__device__ __forceinline__ bool project_or_defer(const ElemLaunch& L, int64_t e, T* hp, T eps)
{
    if constexpr (DeflatedProjection<N>::value)
    {
        const int r = project_translation_deflated<d, N, T, KnownInvariant>(hp, eps);
        if (r < 0) { defer_projection(L, e); return false; }
        return r > 0;
    }
    else return project_positive_definite<d * N, T>(hp, eps);
}

/* element block layout (NP vertex-pair blocks of d x d, row-major) <->
   packed upper triangle of the k x k element Hessian */
template <int d, int N, typename T>
__device__ __forceinline__ void blocks_to_packed(const T* hb, T* h)
{
    constexpr int k = d * N;
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
        for (int b = a; b < N; ++b)
#pragma unroll
            for (int p = 0; p < d; ++p)
#pragma unroll
                for (int q = 0; q < d; ++q)
                {
                    const int i = a * d + p, j = b * d + q;
                    if (i <= j) h[packed_index(i, j, k)] = hb[packed_index(a, b, N) * d * d + p * d + q];
                }
}

template <int d, int N, typename T>
__device__ __forceinline__ void packed_to_blocks(const T* h, T* hb)
{
    constexpr int k = d * N;
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
        for (int b = a; b < N; ++b)
#pragma unroll
            for (int p = 0; p < d; ++p)
#pragma unroll
                for (int q = 0; q < d; ++q)
                {
                    const int i = a * d + p, j = b * d + q;
                    hb[packed_index(a, b, N) * d * d + p * d + q] = (i <= j) ? h[packed_index(i, j, k)] : h[packed_index(j, i, k)];
                }
}

/* Translation-invariant energies (IsTranslationInvariant) with N >= 2 are
   differentiated with respect to slots 1..N-1 only (d(N-1) derivatives,
   slot 0 passive); the full derivatives follow from E(x + t) = E(x):
     g_0 = -sum_{s>=1} g_s,  H_0t = -sum_{s>=1} H_st,  H_00 = sum_{s,t>=1} H_st.
   For a triangle in 2D that is 4 instead of 6 gradient and 10 instead of 21
   Hessian entries per live intermediate (tetrahedron: 9 / 45 instead of
   12 / 78), which is most of the evaluation's work and registers. */
/* a gradient entry as a double-float pair */
__device__ __forceinline__ DoubleFloatValue gf_pair(const DoubleFloat& g) { return DoubleFloatValue(g.hi, g.lo); }
__device__ __forceinline__ DoubleFloatValue gf_pair(double g) { return DoubleFloatValue(g); }

template <typename Energy, int N> struct ReducedDerivatives
{
    static constexpr bool value = IsTranslationInvariant<Energy>::value && N >= 2;
};

template <int d, int N, typename S, typename G, typename T>
__device__ __forceinline__ void lift_translation_invariant(const S& r, G (&g)[d * N], T (&h)[d * N * (d * N + 1) / 2])
{
    constexpr int k = d * N, kr = d * (N - 1);
#pragma unroll
    for (int i = 0; i < d; ++i)
    {
        G acc = G(0);
#pragma unroll
        for (int sl = 1; sl < N; ++sl)
        {
            g[sl * d + i] = r.grad[(sl - 1) * d + i];
            acc = acc + r.grad[(sl - 1) * d + i];
        }
        g[i] = -acc;
    }
    // C[p][J] = sum_{s>=1} H'((s-1)d + p, J): the slot-0 rows, negated
    T C[d][kr];
#pragma unroll
    for (int p = 0; p < d; ++p)
#pragma unroll
        for (int J = 0; J < kr; ++J)
        {
            T acc = T(0);
#pragma unroll
            for (int sl = 1; sl < N; ++sl) acc += r.H((sl - 1) * d + p, J);
            C[p][J] = acc;
        }
#pragma unroll
    for (int I = 0; I < k; ++I)
#pragma unroll
        for (int J = I; J < k; ++J)
        {
            const int a = I / d, p = I % d, b = J / d, q = J % d;
            T v;
            if (a >= 1) v = r.H(I - d, J - d);
            else if (b >= 1) v = -C[p][J - d];
            else
            {
                v = T(0);
#pragma unroll
                for (int t = 1; t < N; ++t) v += C[p][(t - 1) * d + q];
            }
            h[packed_index(I, J, k)] = v;
        }
}

/* Minimum resident 128-thread blocks per SM for k_elem_hessian: 4 (<= 128
   registers) for the FP32-Hessian kernels up to k = 8 -- the reduced k = 6
   mixed kernel needs 168 registers unbounded, spills 72 B at 128, and
   measured 4.7 % faster at the higher occupancy (1.64M-face disk); no bound
   otherwise. */
template <int k, typename T> struct ElemHessianMinBlocks { static constexpr int value = (k <= 8 && sizeof(T) == 4) ? 4 : 1; };

template <int d, int N, typename T, typename Energy>
__global__ void __launch_bounds__(128, ElemHessianMinBlocks<d * N, T>::value) k_elem_hessian(ElemLaunch L, Energy energy)
{
    constexpr int k = d * N;
    constexpr int NP = N * (N + 1) / 2;
    constexpr bool reduced = ReducedDerivatives<Energy, N>::value;
    constexpr int kd = reduced ? d * (N - 1) : k;
    using G = typename GradOf<T, kd>::type;
    using S = Scalar<kd, T, true, typename ValOf<T, k>::type, G>;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= L.n_elem || (L.active && *L.active == 0)) return;
    ActiveElement<d, N, S, reduced> el;
    el.handle = e;
    el.x = L.x;
    el.err = L.err;
#pragma unroll
    for (int i = 0; i < N; ++i) el.vh[i] = L.rec[e * N + i];
    const S r = energy(el);
    G gf[k];
    T hf[k * (k + 1) / 2];
    if constexpr (reduced) lift_translation_invariant<d, N>(r, gf, hf);
    else
    {
#pragma unroll
        for (int i = 0; i < k; ++i) gf[i] = r.grad[i];
#pragma unroll
        for (int i = 0; i < k * (k + 1) / 2; ++i) hf[i] = r.hess[i];
    }
    if (FusedProjection<k>::value && L.project) project_or_defer<d, N, T, reduced>(L, e, hf, (T)L.eps);
    L.out_f[e] = (double)r.val;
    bool fin = true;
    if constexpr (std::is_same<T, float>::value)
    {
        // double-float pairs (the gradient type's own, or split from double)
        float gp[2 * k];
#pragma unroll
        for (int i = 0; i < k; ++i)
        {
            const DoubleFloatValue v = gf_pair(gf[i]);
            gp[2 * i] = v.hi;
            gp[2 * i + 1] = v.lo;
            fin = fin && finite_val(v.hi);
        }
        store_row<float, 2 * k>((float*)L.out_g, e, gp);
    }
    else
    {
        double gv[k];
#pragma unroll
        for (int i = 0; i < k; ++i) { gv[i] = (double)gf[i]; fin = fin && finite_val(gv[i]); }
        store_row<double, k>((double*)L.out_g, e, gv);
    }
    T hb[NP * d * d];
    packed_to_blocks<d, N, T>(hf, hb);
#pragma unroll
    for (int i = 0; i < NP * d * d; ++i) fin = fin && finite_val(hb[i]);
    store_row<T, NP * d * d>((T*)L.out_H, e, hb);
    if (!fin) report_error(L.err, DEVERR_NONFINITE);
}

/* Projection of the element blocks (layout of k_elem_hessian: NP vertex-pair
   blocks of d x d, row-major) in place, one element per thread. */
template <int d, int N, typename T, bool KnownInvariant = false>
__global__ void __launch_bounds__(128) k_project_blocks(ElemLaunch L, T eps)
{
    constexpr int k = d * N;
    constexpr int BS = N * (N + 1) / 2 * d * d;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= L.n_elem || (L.active && *L.active == 0)) return;
    T* Hblocks = (T*)L.out_H;
    T hb[BS];
    load_row<T, BS>(Hblocks, e, hb);
    T h[k * (k + 1) / 2];
    blocks_to_packed<d, N, T>(hb, h);
    if (!project_or_defer<d, N, T, KnownInvariant>(L, e, h, eps)) return;
    packed_to_blocks<d, N, T>(h, hb);
    store_row<T, BS>(Hblocks, e, hb);
}

/* General projection (project_positive_definite<d*N>) of the elements listed
   by project_or_defer, grid-stride over the list. */
template <int d, int N, typename T>
__global__ void __launch_bounds__(128) k_project_general(const uint32_t* __restrict__ list, T* __restrict__ Hblocks, T eps)
{
    constexpr int k = d * N;
    constexpr int BS = N * (N + 1) / 2 * d * d;
    const uint32_t n = list[0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const int64_t e = list[1 + i];
        T hb[BS];
        load_row<T, BS>(Hblocks, e, hb);
        T h[k * (k + 1) / 2];
        blocks_to_packed<d, N, T>(hb, h);
        if (!project_positive_definite<k, T>(h, eps)) continue;
        packed_to_blocks<d, N, T>(h, hb);
        store_row<T, BS>(Hblocks, e, hb);
    }
}

/* ---------------------------------------------------------------------------
 * Lane-split second-order evaluation, mixed precision, for translation-
 * invariant energies with 9 reduced derivatives (d (N - 1) = 9: the
 * tetrahedron, d = 3, N = 4).  The dense kernel above holds a Scalar<9> of
 * 65 registers per live intermediate (FP64 value and gradient, 45-entry FP32
 * Hessian); the symmetric Dirichlet tetrahedron keeps about twenty alive and
 * spilled 5.7 KB a thread.  Here several lanes evaluate each element, each
 * with a 3-derivative scalar (SubsetElement seeds its index triple):
 *   k_elem_grad_lanes  3 lanes per element; lane s: Scalar<3> without
 *                      Hessian, double-float value and gradient, on the
 *                      reduced indices 3s .. 3s+2 -- the energy and the
 *                      accurate gradient;
 *   k_elem_hess_lanes  12 lanes per element; lane l: FP32 Scalar<3> on the
 *                      l-th line of the affine plane of order 3 (points
 *                      (u, c) <-> reduced index 3u + c; every pair of the 9
 *                      indices lies on exactly one of its 12 lines, and the
 *                      3 lines of direction 0 partition them), so the 12
 *                      principal 3 x 3 blocks hold every Hessian entry once.
 * The Hessian lanes evaluate in FP32 (the Hessian's precision), on vertex
 * positions taken relative to the element's first vertex (exact-rounded
 * edge vectors; the energy is translation invariant); the energy and
 * gradient the Newton loop and the line search use come from the
 * double-float lanes.  The blocks are assembled in shared memory, lifted to
 * the first vertex (lift_translation_invariant's sums) and written as one
 * coalesced range; the PSD projection is k_project_blocks (KnownInvariant).
 * Measured on the 48^3 tetrahedral cube (663,552 tets), one projected
 * evaluation: the dense kernel with its fused projection 6.65 ms; here the
 * Hessian lanes 1.2 ms, the gradient lanes 1.1 ms and k_project_blocks
 * 1.0 ms, 3.4 ms in all.  Staging the FP32 relative positions once per
 * element (instead of an FP64 difference and conversion per coordinate and
 * lane) took the Hessian lanes from 1.32 to 1.2 ms.
 * ------------------------------------------------------------------------ */
template <int d, int N, typename T, typename Energy> struct LaneHessian
{
    static constexpr bool value = std::is_same<T, float>::value && ReducedDerivatives<Energy, N>::value && d * (N - 1) == 9;
};

constexpr int GL_ELEMS = 32;   // elements per block of k_elem_grad_lanes (3 lanes each)
constexpr int HL_ELEMS = 8;    // elements per block of k_elem_hess_lanes (12 lanes each)
/* Minimum resident 96-thread blocks per SM of the two kernels: 5, i.e. at
   most 128 registers a thread.  The gradient lanes then keep 984 B of
   spill and the Hessian lanes 112 B; measured on the 48^3 cube (projected
   evaluation with both kernels): 3.52 ms at 5 / 5, 3.72 ms with 168
   registers for the gradient lanes (316 B of spill), and unbounded (255
   registers) they ran slower still -- occupancy pays more than the spill. */
constexpr int GL_MIN_BLOCKS = 5;
constexpr int HL_MIN_BLOCKS = 5;

template <int d, int N, typename Energy>
__global__ void __launch_bounds__(3 * GL_ELEMS, GL_MIN_BLOCKS) k_elem_grad_lanes(ElemLaunch L, Energy energy)
{
    constexpr int k = d * N;
    static_assert(d * (N - 1) == 9, "9 reduced derivatives");
    using S = Scalar<3, float, false, DoubleFloatValue, DoubleFloat>;
    __shared__ float gs[GL_ELEMS][2 * k];   // the element gradient as double-float pairs (hi, lo)
    if (L.active && *L.active == 0) return;
    const int le = threadIdx.x / 3, s = threadIdx.x % 3;
    const int64_t e0 = (int64_t)blockIdx.x * GL_ELEMS, e = e0 + le;
    if (e < L.n_elem)
    {
        SubsetElement<d, N, S, true> el;
        el.handle = e;
        el.x = L.x;
        el.err = L.err;
#pragma unroll
        for (int i = 0; i < N; ++i) el.vh[i] = L.rec[e * N + i];
#pragma unroll
        for (int c = 0; c < 3; ++c) el.idx[c] = 3 * s + c;
        const S r = energy(el);
#pragma unroll
        for (int c = 0; c < 3; ++c)
        {
            gs[le][2 * (d + 3 * s + c)] = r.grad[c].hi;
            gs[le][2 * (d + 3 * s + c) + 1] = r.grad[c].lo;
        }
        if (s == 0) L.out_f[e] = (double)r.val;
    }
    __syncthreads();
    if (e < L.n_elem)
        for (int i = s; i < d; i += 3)
        {
            // first vertex: g_0 = -sum_{slots >= 1} g_slot (lift_translation_invariant)
            DoubleFloat acc(gs[le][2 * (d + i)], gs[le][2 * (d + i) + 1]);
#pragma unroll
            for (int sl = 2; sl < N; ++sl) acc = acc + DoubleFloat(gs[le][2 * (sl * d + i)], gs[le][2 * (sl * d + i) + 1]);
            gs[le][2 * i] = -acc.hi;
            gs[le][2 * i + 1] = -acc.lo;
        }
    __syncthreads();
    const int64_t ne = L.n_elem - e0 < GL_ELEMS ? L.n_elem - e0 : GL_ELEMS;
    float* dst = (float*)L.out_g + e0 * (2 * k);
    bool fin = true;
    for (int q = threadIdx.x; q < ne * 2 * k; q += blockDim.x)
    {
        const float v = gs[q / (2 * k)][q % (2 * k)];
        dst[q] = v;
        fin = fin && finite_val(v);
    }
    if (!fin) report_error(L.err, DEVERR_NONFINITE);
}

/* runs after k_elem_grad_lanes: an element whose energy is not finite (an
   inverted element's +inf) gets a zero Hessian, as the functor's constant
   return gives in the other kernels */
template <int d, int N, typename Energy>
__global__ void __launch_bounds__(12 * HL_ELEMS, HL_MIN_BLOCKS) k_elem_hess_lanes(ElemLaunch L, Energy energy)
{
    constexpr int k = d * N, R = d * (N - 1), NR = R * (R + 1) / 2;
    constexpr int BS = N * (N + 1) / 2 * d * d;
    static_assert(R == 9, "9 reduced derivatives");
    using S = Scalar<3, float, true, float, float>;
    __shared__ float xsh[HL_ELEMS][k];      // positions relative to the first vertex, FP32
    __shared__ float hr[HL_ELEMS][NR];      // packed reduced Hessian per element
    __shared__ float cs[HL_ELEMS][d][R];    // its slot-0 row sums C[p][J] = sum_s Hr(s d + p, J)
    __shared__ bool inf_e[HL_ELEMS];        // the element's energy is not finite
    if (L.active && *L.active == 0) return;
    const int le = threadIdx.x / 12, l = threadIdx.x % 12;
    const int64_t e0 = (int64_t)blockIdx.x * HL_ELEMS, e = e0 + le;
    auto Hr = [&](int ei, int i, int j) { return i <= j ? hr[ei][packed_index(i, j, R)] : hr[ei][packed_index(j, i, R)]; };
    SubsetElement<d, N, S, true, true> el;
    if (e < L.n_elem)
    {
#pragma unroll
        for (int i = 0; i < N; ++i) el.vh[i] = L.rec[e * N + i];
        // the element's positions relative to its first vertex, one coordinate
        // per lane (the lanes of an element share them)
        for (int q = l; q < k; q += 12)
        {
            const int sl = q / d, c = q % d;
            const int32_t v0 = el.vh[0], v = el.vh[sl] >= 0 ? el.vh[sl] : v0;   // -1: slot not recorded
            xsh[le][q] = v0 < 0 ? 0.f : (float)(L.x[(int64_t)d * v + c] - L.x[(int64_t)d * v0 + c]);
        }
    }
    __syncthreads();
    if (e < L.n_elem)
    {
        el.handle = e;
        el.x = L.x;
        el.err = L.err;
        el.xs = xsh[le];
        plane_line(l, el.idx);
        const S r = energy(el);
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int q = p; q < 3; ++q)
                if (q > p || l < 3)   // diagonal entries from the direction-0 lines only
                {
                    const int I = el.idx[p], J = el.idx[q];
                    hr[le][I <= J ? packed_index(I, J, R) : packed_index(J, I, R)] = r.H(p, q);
                }
        if (l == 0) inf_e[le] = !finite_val(L.out_f[e]);
    }
    __syncthreads();
    const int64_t ne = L.n_elem - e0 < HL_ELEMS ? L.n_elem - e0 : HL_ELEMS;
    for (int q = threadIdx.x; q < ne * d * R; q += blockDim.x)
    {
        // lift_translation_invariant's sums: H_0t = -C, H_00 = sum over the C blocks
        const int ei = q / (d * R), p = (q / R) % d, J = q % R;
        float acc = 0.f;
#pragma unroll
        for (int sl = 0; sl < N - 1; ++sl) acc += Hr(ei, sl * d + p, J);
        cs[ei][p][J] = acc;
    }
    __syncthreads();
    float* dst = (float*)L.out_H + e0 * BS;
    bool fin = true;
    for (int q = threadIdx.x; q < ne * BS; q += blockDim.x)
    {
        const int ei = q / BS, w = q % BS;
        int P = w / (d * d);   // vertex pair (a, b), a <= b, in packed order
        const int pp = (w % (d * d)) / d, qq = w % d;
        int a = 0;
        while (P >= N - a) { P -= N - a; ++a; }
        const int b = a + P;
        float v;
        if (a >= 1) v = Hr(ei, (a - 1) * d + pp, (b - 1) * d + qq);
        else if (b >= 1) v = -cs[ei][pp][(b - 1) * d + qq];
        else
        {
            v = 0.f;
#pragma unroll
            for (int t = 0; t < N - 1; ++t) v += cs[ei][pp][t * d + qq];
        }
        if (inf_e[ei]) v = 0.f;
        dst[q] = v;
        fin = fin && finite_val(v);
    }
    if (!fin) report_error(L.err, DEVERR_NONFINITE);
}

inline unsigned elem_grid(int64_t n) { return (unsigned)((n + 127) / 128); }

/* ElemLaunch from the C-ABI callback arguments */
inline ElemLaunch make_launch(const tad_term_eval_args& a)
{
    ElemLaunch L{};
    L.n_elem = a.n_elem;
    L.rec = a.handles_d;
    L.x = a.x_d;
    L.dir = a.dir_d;
    L.steps = a.steps_d;
    L.n_steps = a.n_steps;
    L.f_stride = a.f_row_stride;
    L.eps = a.proj_eps;
    L.project = a.mode == 3;
    L.out_f = (double*)a.out_f_d;
    L.out_g = a.out_g_d;
    L.out_H = a.out_H_d;
    L.record = a.record_d;
    L.err = a.error_d;
    L.out_r = a.out_r_d;
    L.out_J = a.out_J_d;
    L.out_Hv = a.out_Hv_d;
    L.proj_list = a.proj_list_d;
    L.active = a.active_d;
    return L;
}

/* Second-order kernels (modes 2, 3) in precision T; split from the others
   so a translation unit can instantiate them alone. */
template <int d, int N, typename T, typename Energy>
inline void launch_elements_hessian(const ElemLaunch& L, const Energy& energy, cudaStream_t s)
{
    if (L.n_elem <= 0) return;
    // energies that declare translation invariance take the deflated form
    // without a test, so they never list an element for the general kernel:
    // neither the list nor that kernel is needed for them
    constexpr bool deflated = DeflatedProjection<N>::value && !ReducedDerivatives<Energy, N>::value;
    if (deflated && L.project && L.proj_list) cudaMemsetAsync(L.proj_list, 0, sizeof(uint32_t), s);
    if constexpr (LaneHessian<d, N, T, Energy>::value)
    {
        k_elem_grad_lanes<d, N, Energy><<<(unsigned)((L.n_elem + GL_ELEMS - 1) / GL_ELEMS), 3 * GL_ELEMS, 0, s>>>(L, energy);
        k_elem_hess_lanes<d, N, Energy><<<(unsigned)((L.n_elem + HL_ELEMS - 1) / HL_ELEMS), 12 * HL_ELEMS, 0, s>>>(L, energy);
        if (L.project) k_project_blocks<d, N, T, true><<<elem_grid(L.n_elem), 128, 0, s>>>(L, (T)L.eps);
        return;
    }
    k_elem_hessian<d, N, T, Energy><<<elem_grid(L.n_elem), 128, 0, s>>>(L, energy);
    if constexpr (!FusedProjection<d * N>::value)
        if (L.project)
            k_project_blocks<d, N, T, ReducedDerivatives<Energy, N>::value><<<elem_grid(L.n_elem), 128, 0, s>>>(L, (T)L.eps);
    if constexpr (deflated)
        if (L.project && L.proj_list)
            k_project_general<d, N, T><<<std::min(elem_grid(L.n_elem), 1216u), 128, 0, s>>>(L.proj_list, (T*)L.out_H, (T)L.eps);
}

/* Value, gradient, line-search and record kernels (modes 0, 1, 4, 5).  The
   line-search energies of mixed precision (precision 1) use the value type
   of the mixed second-order kernel, so that the Armijo test compares f(x)
   and f(x + s d) computed alike. */
template <int d, int N, typename Energy>
inline void launch_elements_first_order(int mode, const ElemLaunch& L, const Energy& energy, cudaStream_t s,
                                        int precision = 0)
{
    if (L.n_elem <= 0) return;
    const unsigned g = elem_grid(L.n_elem);
    // the value type of the mixed second-order kernels (double-float for the lane-split ones)
    using PMixed = std::conditional_t<LaneHessian<d, N, float, Energy>::value, DoubleFloatValue,
                                      typename ValOf<float, d * N>::type>;
    switch (mode)
    {
    case 0: k_elem_value<d, N, Energy><<<g, 128, 0, s>>>(L, energy); break;
    case 1: k_elem_gradient<d, N, Energy><<<g, 128, 0, s>>>(L, energy); break;
    case 4:
        if (precision == 1) k_elem_linesearch<d, N, Energy, PMixed><<<g, 128, 0, s>>>(L, energy);
        else k_elem_linesearch<d, N, Energy, double><<<g, 128, 0, s>>>(L, energy);
        break;
    case 5: k_elem_record<d, N, Energy><<<g, 128, 0, s>>>(L, energy); break;
    }
}

/* Launch the kernel for `mode` (tad_eval_mode values) on stream s. */
template <int d, int N, typename Energy>
inline void launch_elements(int mode, int precision, const ElemLaunch& L, const Energy& energy, cudaStream_t s)
{
    if (mode == 2 || mode == 3)
    {
        if (precision == 1) launch_elements_hessian<d, N, float>(L, energy, s);
        else launch_elements_hessian<d, N, double>(L, energy, s);
    }
    else launch_elements_first_order<d, N>(mode, L, energy, s, precision);
}

/* ---------------------------------------------------------------------------
 * Vector functors (VectorFunction, include/TinyAD/Detail/VectorObjectiveTerm.hh):
 * the functor returns tad::Vec<T, M>, M residuals per element.  The scalar
 * modes evaluate the sum of squares f_e = sum_o r_o^2 (VALUE, LINESEARCH),
 * its gradient 2 sum_o r_o grad r_o (GRADIENT) and the Gauss-Newton blocks
 * 2 sum_o grad r_o grad r_o^T (HESSIAN, HESSIAN_PROJ; PSD, written as the
 * vertex-pair blocks the assembly of scalar terms reads).  VEC_JACOBIAN adds
 * the residuals and their gradients in local slot order, VEC_DERIVATIVES also
 * the packed residual Hessians.  FP64 (the Gauss-Newton blocks are written
 * in the problem's Hessian precision T).
 * ------------------------------------------------------------------------ */
template <int d, int N, int M, typename Energy>
__global__ void __launch_bounds__(128) k_vec_value(ElemLaunch L, Energy energy)
{
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= L.n_elem) return;
    PassiveElement<d, N, double> el{e, L.x};
    const Vec<double, M> r = energy(el);
    double f = 0.0;
#pragma unroll
    for (int o = 0; o < M; ++o)
    {
        f += r[o] * r[o];
        if (L.out_r) L.out_r[e * M + o] = r[o];
    }
    L.out_f[e] = f;
}

template <int d, int N, int M, typename Energy>
__global__ void __launch_bounds__(128) k_vec_linesearch(ElemLaunch L, Energy energy)
{
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= L.n_elem || (L.active && *L.active == 0)) return;
    for (int j = 0; j < L.n_steps; ++j)
    {
        LineSearchElement<d, N, double> el{e, L.x, L.dir, L.steps[j]};
        const Vec<double, M> r = energy(el);
        double f = 0.0;
#pragma unroll
        for (int o = 0; o < M; ++o) f += r[o] * r[o];
        L.out_f[(int64_t)j * L.f_stride + e] = f;
    }
}

/* first order: f, g = 2 J^T r, optionally r and J, optionally the
   Gauss-Newton blocks (gn) in precision T */
template <int d, int N, int M, typename T, typename Energy>
__global__ void __launch_bounds__(128) k_vec_first_order(ElemLaunch L, Energy energy, bool gn)
{
    constexpr int k = d * N;
    constexpr int NP = N * (N + 1) / 2;
    using S = Scalar<k, double, false>;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= L.n_elem || (L.active && *L.active == 0)) return;
    ActiveElement<d, N, S> el;
    el.handle = e;
    el.x = L.x;
    el.err = L.err;
#pragma unroll
    for (int i = 0; i < N; ++i) el.vh[i] = L.rec[e * N + i];
    const Vec<S, M> r = energy(el);
    double f = 0.0, g[k];
    bool fin = true;
#pragma unroll
    for (int i = 0; i < k; ++i) g[i] = 0.0;
#pragma unroll
    for (int o = 0; o < M; ++o)
    {
        const double ro = r[o].val;
        f += ro * ro;
        if (L.out_r) L.out_r[e * M + o] = ro;
#pragma unroll
        for (int i = 0; i < k; ++i)
        {
            g[i] += 2.0 * ro * r[o].grad[i];
            fin = fin && finite_val(r[o].grad[i]);
            if (L.out_J) L.out_J[(e * M + o) * k + i] = r[o].grad[i];
        }
    }
    L.out_f[e] = f;
    if (gn && std::is_same<T, float>::value)
    {
        // mixed second-order mode: double-float pairs, as k_elem_hessian writes them
        float gp[2 * k];
#pragma unroll
        for (int i = 0; i < k; ++i)
        {
            const DoubleFloatValue v(g[i]);
            gp[2 * i] = v.hi;
            gp[2 * i + 1] = v.lo;
        }
        store_row<float, 2 * k>((float*)L.out_g, e, gp);
    }
    else store_row<double, k>((double*)L.out_g, e, g);
    if (gn)
    {
        T hb[NP * d * d];
#pragma unroll
        for (int a = 0; a < N; ++a)
#pragma unroll
            for (int b = a; b < N; ++b)
#pragma unroll
                for (int p = 0; p < d; ++p)
#pragma unroll
                    for (int q = 0; q < d; ++q)
                    {
                        const int i = a * d + p, j = b * d + q;
                        double acc = 0.0;
#pragma unroll
                        for (int o = 0; o < M; ++o) acc += r[o].grad[i] * r[o].grad[j];
                        hb[packed_index(a, b, N) * d * d + p * d + q] = (T)(2.0 * acc);
                    }
        store_row<T, NP * d * d>((T*)L.out_H, e, hb);
    }
    if (!fin) report_error(L.err, DEVERR_NONFINITE);
}

/* second order: r, J and the packed residual Hessians */
template <int d, int N, int M, typename Energy>
__global__ void __launch_bounds__(128) k_vec_second_order(ElemLaunch L, Energy energy)
{
    constexpr int k = d * N;
    constexpr int NH = k * (k + 1) / 2;
    using S = Scalar<k, double, true>;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= L.n_elem) return;
    ActiveElement<d, N, S> el;
    el.handle = e;
    el.x = L.x;
    el.err = L.err;
#pragma unroll
    for (int i = 0; i < N; ++i) el.vh[i] = L.rec[e * N + i];
    const Vec<S, M> r = energy(el);
    double f = 0.0;
#pragma unroll
    for (int o = 0; o < M; ++o)
    {
        f += r[o].val * r[o].val;
        if (L.out_r) L.out_r[e * M + o] = r[o].val;
#pragma unroll
        for (int i = 0; i < k; ++i)
            if (L.out_J) L.out_J[(e * M + o) * k + i] = r[o].grad[i];
#pragma unroll
        for (int q = 0; q < NH; ++q)
            if (L.out_Hv) L.out_Hv[(e * M + o) * NH + q] = r[o].hess[q];
    }
    L.out_f[e] = f;
}

/* Launch the vector-term kernel for `mode` on stream s. */
template <int d, int N, int M, typename Energy>
inline void launch_vector_elements(int mode, int precision, const ElemLaunch& L, const Energy& energy, cudaStream_t s)
{
    if (L.n_elem <= 0) return;
    const unsigned g = elem_grid(L.n_elem);
    switch (mode)
    {
    case 0: k_vec_value<d, N, M, Energy><<<g, 128, 0, s>>>(L, energy); break;
    case 4: k_vec_linesearch<d, N, M, Energy><<<g, 128, 0, s>>>(L, energy); break;
    case 5: k_elem_record<d, N, Energy><<<g, 128, 0, s>>>(L, energy); break;
    case 1:
    case 6: k_vec_first_order<d, N, M, double, Energy><<<g, 128, 0, s>>>(L, energy, false); break;
    case 2:
    case 3:
        if (precision == 1) k_vec_first_order<d, N, M, float, Energy><<<g, 128, 0, s>>>(L, energy, true);
        else k_vec_first_order<d, N, M, double, Energy><<<g, 128, 0, s>>>(L, energy, true);
        break;
    case 7: k_vec_second_order<d, N, M, Energy><<<g, 128, 0, s>>>(L, energy); break;
    }
}

} // namespace tad
