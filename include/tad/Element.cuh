/*
 * tad/Element.cuh -- what an element functor receives: `element.handle` and
 * `element.variables(vh)` (include/TinyAD/Detail/Element.hh:93-144).
 *
 * The reference builds each element's local index map on every call, in
 * first-access order with de-duplication (Element.hh:208-260).  Here the map
 * is recorded once, when the sparsity pattern is built (RecordElement), and
 * every later evaluation looks the handle up in the element's recorded list
 * of at most N handles held in registers: the local index of handle vh is
 * d * (its position in that list) + i, exactly the reference's order.
 *
 * Element kinds:
 *   ActiveElement<d, N, S>   seeds tad::Scalar variables (gradient/Hessian)
 *   PassiveElement<d, N, T>  returns plain values (energy only)
 *   LineSearchElement<d, N>  returns x + s * dir (passive, line search)
 *   RecordElement<d, N>      records the first-access order
 */
#pragma once
#include <stdint.h>
#include <type_traits>
#include "Mat.cuh"

namespace tad {

/* device error word bits */
enum : int32_t {
    DEVERR_UNRECORDED_ACCESS = 1,   /* handle not in the recorded access list */
    DEVERR_TOO_MANY_VARS = 2,       /* more distinct handles than the valence */
    DEVERR_NONFINITE = 4,           /* non-finite gradient/Hessian entry */
    DEVERR_TIMEOUT = 8,             /* bounded wait gave up */
    DEVERR_NO_PROJ_LIST = 16        /* HESSIAN_PROJ launched without the projection list */
};

#if defined(__CUDACC__)
__device__ __forceinline__ void report_error(int32_t* err, int32_t bit)
{
    if (err) atomicOr(err, bit);
}
#endif

/* FirstPassive: the first recorded vertex (slot 0) enters as a constant and
   slot s >= 1 seeds derivative indices (s-1)*d + i, so S has d(N-1)
   derivatives -- for translation-invariant energies, whose slot-0
   derivatives follow from the others (lift_translation_invariant). */
template <int d, int N, typename S, bool FirstPassive = false>
struct ActiveElement
{
    using scalar_type = S;
    using passive_type = typename S::passive_type;
    static constexpr bool active_mode = true;
    int64_t handle;
    int32_t vh[N];
    const double* x;
    int32_t* err;

    TAD_HD int slot_of(int v) const
    {
        int slot = -1;
#pragma unroll
        for (int i = N - 1; i >= 0; --i)
            if (vh[i] == v) slot = i;
        return slot;
    }

#if defined(__CUDACC__)
    __device__ Vec<S, d> variables(int v) const
    {
        int slot = slot_of(v);
        if (slot < 0) { report_error(err, DEVERR_UNRECORDED_ACCESS); slot = 0; }
        Vec<S, d> r;
#pragma unroll
        for (int i = 0; i < d; ++i) r[i] = S((passive_type)x[(int64_t)d * v + i], (FirstPassive ? slot - 1 : slot) * d + i);
        return r;
    }
    __device__ S variable(int v) const
    {
        static_assert(d == 1, "element.variable(vh) needs variable dimension 1; use element.variables(vh)");
        return variables(v)[0];
    }
#endif
};

/* An ActiveElement whose scalar S carries only m = S::k of the element's
   derivatives: variable j of the derivative numbering above (FirstPassive:
   j = (slot - 1) * d + i) becomes local derivative p of S when idx[p] == j,
   and enters as a constant otherwise.  S's Hessian is then the m x m
   principal block of the element Hessian on the indices idx, and its
   gradient those m gradient entries; lanes evaluating one element with
   index sets that cover every index pair together obtain the whole Hessian
   (k_elem_hess_lanes, ElementKernels.cuh).  Staged: the positions come from
   xs (slot-major, d per recorded vertex, already in the passive type), which
   the lanes of one element fill together -- the lane-split kernel stages
   them relative to the first vertex (translation-invariant energies), so an
   FP32 evaluation sees exact-rounded edge vectors. */
template <int d, int N, typename S, bool FirstPassive = false, bool Staged = false>
struct SubsetElement
{
    using scalar_type = S;
    using passive_type = typename S::passive_type;
    static constexpr bool active_mode = true;
    int64_t handle;
    int32_t vh[N];
    int idx[S::k];
    const double* x;
    int32_t* err;
    const passive_type* xs;

    TAD_HD Vec<S, d> variables(int v) const
    {
        int slot = -1;
#pragma unroll
        for (int i = N - 1; i >= 0; --i)
            if (vh[i] == v) slot = i;
        if (slot < 0)
        {
#if defined(__CUDA_ARCH__)
            report_error(err, DEVERR_UNRECORDED_ACCESS);
#endif
            slot = 0;
        }
        Vec<S, d> r;
#pragma unroll
        for (int i = 0; i < d; ++i)
        {
            S s(Staged ? xs[slot * d + i] : (passive_type)x[(int64_t)d * v + i]);
            const int j = (FirstPassive ? slot - 1 : slot) * d + i;
#pragma unroll
            for (int p = 0; p < S::k; ++p)
                if (idx[p] == j) s.grad[p] = typename S::grad_type(1);
            r[i] = s;
        }
        return r;
    }
    TAD_HD S variable(int v) const
    {
        static_assert(d == 1, "element.variable(vh) needs variable dimension 1; use element.variables(vh)");
        return variables(v)[0];
    }
};

/* Index triple of line l (0..11) of the affine plane of order 3, on the 9
   indices 3u + c (points (u, c), u, c in 0..2): the lines of direction 0 are
   {3u, 3u+1, 3u+2}; those of slope a = dir - 1 through (0, c) are
   {(u, c + a u mod 3)}.  Any two points lie on exactly one line, so the 12
   lines' 3 x 3 principal blocks hold every off-diagonal entry of a 9 x 9
   matrix once, and the 3 lines of direction 0 hold each diagonal entry once
   (k_elem_hess_lanes; tests/cpp/lane_split_test.cpp checks both). */
TAD_HD void plane_line(int l, int (&t)[3])
{
    const int dir = l / 3, c = l % 3;
    if (dir == 0) { t[0] = 3 * c; t[1] = 3 * c + 1; t[2] = 3 * c + 2; }
    else
    {
        const int a = dir - 1;   // slope
        t[0] = c;
        t[1] = 3 + (c + a) % 3;
        t[2] = 6 + (c + 2 * a) % 3;
    }
}

template <int d, int N, typename T>
struct PassiveElement
{
    using scalar_type = T;
    using passive_type = T;
    static constexpr bool active_mode = false;
    int64_t handle;
    const double* x;

    TAD_HD Vec<T, d> variables(int v) const
    {
        Vec<T, d> r;
#pragma unroll
        for (int i = 0; i < d; ++i) r[i] = (T)x[(int64_t)d * v + i];
        return r;
    }
    TAD_HD T variable(int v) const { return variables(v)[0]; }
};

template <int d, int N, typename P = double>
struct LineSearchElement
{
    using scalar_type = P;
    using passive_type = P;
    static constexpr bool active_mode = false;
    int64_t handle;
    const double* x;
    const double* dir;
    P s;

    /* trial point x + s dir in the passive type P (double, or the
       double-float of mixed mode, where it is formed without FP64 work) */
    TAD_HD Vec<P, d> variables(int v) const
    {
        Vec<P, d> r;
#pragma unroll
        for (int i = 0; i < d; ++i) r[i] = P(x[(int64_t)d * v + i]) + s * P(dir[(int64_t)d * v + i]);
        return r;
    }
    TAD_HD P variable(int v) const { return variables(v)[0]; }
};

template <int d, int N>
struct RecordElement
{
    using scalar_type = double;
    using passive_type = double;
    static constexpr bool active_mode = false;
    int64_t handle;
    const double* x;
    int32_t vh[N];
    int n = 0;
    bool overflow = false;

    TAD_HD Vec<double, d> variables(int v)
    {
        bool seen = false;
#pragma unroll
        for (int i = 0; i < N; ++i)
            if (i < n && vh[i] == v) seen = true;
        if (!seen)
        {
            if (n < N) vh[n++] = v;
            else overflow = true;
        }
        Vec<double, d> r;
#pragma unroll
        for (int i = 0; i < d; ++i) r[i] = x[(int64_t)d * v + i];
        return r;
    }
    TAD_HD double variable(int v) { return variables(v)[0]; }
};

/* TINYAD_SCALAR_TYPE(element) of the reference (Element.hh:300-331) */
/* Energies invariant under a common translation of all their vertices
   declare `static constexpr bool translation_invariant = true;` (a function
   of edge vectors / vertex differences only).  The second-order kernels then
   differentiate with respect to N-1 vertices and recover the first one's
   derivatives from the invariance, and the PSD projection works on the
   d(N-1)-dimensional complement of the translations. */
template <typename E, typename = void> struct IsTranslationInvariant : std::false_type {};
template <typename E>
struct IsTranslationInvariant<E, std::void_t<decltype(E::translation_invariant)>>
    : std::integral_constant<bool, E::translation_invariant> {};

#define TAD_SCALAR_TYPE(element) typename std::decay_t<decltype(element)>::scalar_type
#define TAD_PASSIVE_TYPE(element) typename std::decay_t<decltype(element)>::passive_type
#define TAD_ACTIVE_MODE(element) (std::decay_t<decltype(element)>::active_mode)

} // namespace tad
