/*
 * Projected-Newton step on the device: linear solve + backtracking line
 * search (the reference's newton_direction, include/TinyAD/Utils/
 * NewtonDirection.hh:25-65, and line_search, include/TinyAD/Utils/
 * LineSearch.hh:14-65, around the loop of tests/NewtonTest.cc:69-75).
 *
 * Linear solve.  The reference factorises H with Eigen's SimplicialLDLT; a
 * serial sparse factorisation has no good GB300 mapping, so d = -(H + wI)^-1 g
 * is solved by preconditioned conjugate gradients with a block-Jacobi
 * preconditioner (inverted d x d diagonal blocks).  One iteration is two
 * kernels over a fixed grid (RED_BLOCKS x RED_THREADS, grid-stride):
 *   k_pcg_spmv_fused  Ap = H z + beta Ap and p = z + beta p (BSR, one thread
 *                     per block row; k_pcg_spmv_vec, 8 lanes per row, for
 *                     3 x 3 blocks), fused with the p.Ap reduction; the last
 *                     block computes alpha on the device
 *   k_pcg_update      x += alpha p, r -= alpha Ap, z = M^-1 r fused with the
 *                     r.z and r.r reductions; the last block computes beta and
 *                     sets the convergence flag (|r| <= tol |b|) or the cap
 * Scalars never leave the device; every kernel returns at once when the flag
 * is set, so chunks of iterations are captured once in a CUDA graph and
 * replayed, with one host check per replay.  Reductions have a fixed order
 * (bitwise reproducible).
 *
 * Mixed precision: H, the PCG vectors and the SpMV are FP32 (dot products are
 * accumulated per thread in FP32 and combined in FP64); an FP64 iterative-
 * refinement loop around it computes r = b - H d with FP64 accumulation and
 * FP64 d, solving the FP32 system for the correction each pass.
 *
 * Line search.  Trial step sizes follow the reference's sequence (s_max,
 * s *= shrink, snap to 1); the energy at x + s d is evaluated for a batch of
 * trials in one launch per term (first batch 1 trial, then LS_BATCH), the
 * first trial meeting the Armijo condition is accepted, as in the
 * reference's sequential loop.
 */
#include <cmath>
#include <vector>

#include "internal.hh"
#include "../../include/tad/Scalar.cuh"
#include "grid_reduce.cuh"
#include "bsr_kernels.cuh"

namespace tadlib {

/* x = 0, r = b, z = M^-1 r, p = Ap = 0, beta = 0 (the first fused SpMV then
   forms p = z, Ap = A z); rz = r.z, bb = b.b.  With H given (block Jacobi),
   the inverted diagonal blocks of H + w I are formed here and stored in dinv;
   with H = NULL dinv is read (the AMG finest level's). */
template <int d, typename T>
__global__ void __launch_bounds__(RED_THREADS) k_pcg_init(int64_t nh, const double* __restrict__ b, T* x, T* r, T* z, T* p,
                                                          T* Ap, T* __restrict__ dinv, const int32_t* __restrict__ diag,
                                                          const T* __restrict__ H, double w, double* partials,
                                                          unsigned* counter, DevScalars* ds, double rel_tol, int max_iters)
{
    // per-thread partials in the PCG's precision (a few rows each), combined in FP64
    T acc_rz = T(0), acc_bb = T(0);
    GRID_STRIDE(u, nh)
    {
        T rv[d], zv[d];
#pragma unroll
        for (int i = 0; i < d; ++i) { rv[i] = from_double<T>(b[u * d + i]); x[u * d + i] = T(0); r[u * d + i] = rv[i]; }
        if (H)
        {
            T I[d * d];
            diag_block_inverse<d, T>(diag, H, w, u, I);
#pragma unroll
            for (int i = 0; i < d; ++i)
            {
                T acc = T(0);
#pragma unroll
                for (int j = 0; j < d; ++j) { acc += I[i * d + j] * rv[j]; dinv[u * d * d + i * d + j] = I[i * d + j]; }
                zv[i] = acc;
            }
        }
        else apply_dinv<d, T>(dinv, u, rv, zv);
#pragma unroll
        for (int i = 0; i < d; ++i)
        {
            z[u * d + i] = zv[i];
            p[u * d + i] = T(0);
            Ap[u * d + i] = T(0);
            acc_rz += rv[i] * zv[i];
            acc_bb += rv[i] * rv[i];
        }
    }
    double part[2] = {as_double(acc_rz), as_double(acc_bb)};
    double tot[2];
    if (!grid_sum<2>(part, partials, counter, tot)) return;
    if (threadIdx.x == 0)
    {
        ds->rz = tot[0];
        ds->bb = tot[1];
        ds->rr = tot[1];
        ds->beta = 0.0;
        ds->tol2 = rel_tol * rel_tol * tot[1];
        ds->iters = 0;
        ds->breakdown = 0;
        ds->done = (tot[1] == 0.0) ? 1 : 0;
        ds->max_iters = max_iters;
    }
}

template <int d, typename T>
__global__ void __launch_bounds__(RED_THREADS) k_pcg_spmv(int64_t nh, const int32_t* __restrict__ bptr, const int32_t* __restrict__ bcol,
                                                          const T* __restrict__ H, const T* __restrict__ p, T* __restrict__ Ap,
                                                          double* partials, unsigned* counter, DevScalars* ds)
{
    if (*(volatile int32_t*)&ds->done) return;
    T part = T(0);
    GRID_STRIDE(u, nh)
    {
        T y[d];
#pragma unroll
        for (int i = 0; i < d; ++i) y[i] = T(0);
        const int32_t b1 = bptr[u + 1];
        for (int32_t b = bptr[u]; b < b1; ++b)
        {
            const int64_t v = bcol[b];
            T pv[d];
#pragma unroll
            for (int j = 0; j < d; ++j) pv[j] = p[v * d + j];
            const T* B = H + (int64_t)b * d * d;
#pragma unroll
            for (int i = 0; i < d; ++i)
#pragma unroll
                for (int j = 0; j < d; ++j) y[i] += B[i * d + j] * pv[j];
        }
#pragma unroll
        for (int i = 0; i < d; ++i)
        {
            Ap[u * d + i] = y[i];
            part += p[u * d + i] * y[i];
        }
    }
    double v[1] = {as_double(part)}, tot[1];
    if (!grid_sum<1>(v, partials, counter, tot)) return;
    if (threadIdx.x == 0)
    {
        ds->pAp = tot[0];
        if (!(tot[0] > 0.0) || !isfinite(tot[0]))
        {
            ds->breakdown = 1;
            ds->done = 1;
            ds->alpha = 0.0;
        }
        else ds->alpha = ds->rz / tot[0];
    }
}

/* SpMV fused with the p update and the p.Ap reduction:
     Ap = A z + beta Ap,  p = z + beta p  (A p_new = A z + beta A p_old),
   so p is never gathered and the separate p = z + beta p pass disappears.
   One thread per block row (bsr_row_product). */
template <int d, typename T, int G>
__global__ void __launch_bounds__(RED_THREADS) k_pcg_spmv_fused(int64_t nh, const int32_t* __restrict__ bptr,
                                                                const int32_t* __restrict__ bcol, const T* __restrict__ H,
                                                                const T* __restrict__ z, T* __restrict__ p, T* __restrict__ Ap,
                                                                double* partials, unsigned* counter, DevScalars* ds)
{
    if (*(volatile int32_t*)&ds->done) return;
    const T beta = from_double<T>(ds->beta);
    T part = T(0);
    GRID_STRIDE(u, nh)
    {
        T y[d];
        bsr_row_product4<d, T>(bptr, bcol, H, z, u, y);
#pragma unroll
        for (int i = 0; i < d; ++i)
        {
            const T apn = y[i] + beta * Ap[u * d + i];
            const T pn = z[u * d + i] + beta * p[u * d + i];
            Ap[u * d + i] = apn;
            p[u * d + i] = pn;
            part += pn * apn;
        }
    }
    double v[1] = {as_double(part)}, tot[1];
    if (!grid_sum<1>(v, partials, counter, tot)) return;
    if (threadIdx.x == 0)
    {
        ds->pAp = tot[0];
        if (!(tot[0] > 0.0) || !isfinite(tot[0]))
        {
            ds->breakdown = 1;
            ds->done = 1;
            ds->alpha = 0.0;
        }
        else ds->alpha = ds->rz / tot[0];
    }
}

/* The same SpMV with L lanes per block row (CSR-vector form): lane l of a
   row's group handles blocks l, l + L, ...; consecutive lanes read
   consecutive blocks and column ids (coalesced), and the partial products
   are summed by xor shuffles within the group.  Warps loop over uniform row
   bases (32 / L rows each), so every lane takes part in every shuffle. */
template <int d, typename T, int L>
__global__ void __launch_bounds__(RED_THREADS) k_pcg_spmv_vec(int64_t nh, const int32_t* __restrict__ bptr,
                                                              const int32_t* __restrict__ bcol, const T* __restrict__ H,
                                                              const T* __restrict__ z, T* __restrict__ p, T* __restrict__ Ap,
                                                              double* partials, unsigned* counter, DevScalars* ds)
{
    static_assert(L >= d && 32 % L == 0, "lanes per row");
    if (*(volatile int32_t*)&ds->done) return;
    const T beta = from_double<T>(ds->beta);
    T part = T(0);
    constexpr int RPW = 32 / L;   // rows per warp pass
    const int lane = threadIdx.x & (L - 1);
    const int sub = (threadIdx.x & 31) / L;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp * RPW; base < nh; base += n_warps * RPW)
    {
        const int64_t u = base + sub;
        T y[d];
#pragma unroll
        for (int i = 0; i < d; ++i) y[i] = T(0);
        if (u < nh)
        {
            const int32_t b1 = bptr[u + 1];
            for (int32_t b = bptr[u] + lane; b < b1; b += L)
            {
                const int64_t v = __ldg(bcol + b);
                T B[d * d], zv[d];
                load_block<d, T>(H + (int64_t)b * d * d, B);
                load_vec<d, T>(z + v * d, zv);
#pragma unroll
                for (int i = 0; i < d; ++i)
#pragma unroll
                    for (int j = 0; j < d; ++j) y[i] += B[i * d + j] * zv[j];
            }
        }
#pragma unroll
        for (int off = L / 2; off > 0; off >>= 1)
#pragma unroll
            for (int i = 0; i < d; ++i) y[i] += __shfl_xor_sync(0xffffffffu, y[i], off, L);
        if (u < nh && lane < d)
        {
            // lane i of the group owns entry i of the row
            T yi = y[0];
#pragma unroll
            for (int i = 1; i < d; ++i) if (lane == i) yi = y[i];
            const int64_t q = u * d + lane;
            const T apn = yi + beta * Ap[q];
            const T pn = z[q] + beta * p[q];
            Ap[q] = apn;
            p[q] = pn;
            part += pn * apn;
        }
    }
    double v[1] = {as_double(part)}, tot[1];
    if (!grid_sum<1>(v, partials, counter, tot)) return;
    if (threadIdx.x == 0)
    {
        ds->pAp = tot[0];
        if (!(tot[0] > 0.0) || !isfinite(tot[0]))
        {
            ds->breakdown = 1;
            ds->done = 1;
            ds->alpha = 0.0;
        }
        else ds->alpha = ds->rz / tot[0];
    }
}

/* k_pcg_spmv_fused on the sliced-ELL copy of H (sell_row_product) */
template <int d, typename T>
__global__ void __launch_bounds__(RED_THREADS) k_pcg_spmv_sell(int64_t nh, const int32_t* __restrict__ sptr,
                                                               const int32_t* __restrict__ scol, const T* __restrict__ Hs,
                                                               const T* __restrict__ z, T* __restrict__ p, T* __restrict__ Ap,
                                                               double* partials, unsigned* counter, DevScalars* ds)
{
    if (*(volatile int32_t*)&ds->done) return;
    const T beta = from_double<T>(ds->beta);
    T part = T(0);
    GRID_STRIDE(u, nh)
    {
        T y[d];
        sell_row_product<d, T>(sptr, scol, Hs, z, u, y);
#pragma unroll
        for (int i = 0; i < d; ++i)
        {
            const T apn = y[i] + beta * Ap[u * d + i];
            const T pn = z[u * d + i] + beta * p[u * d + i];
            Ap[u * d + i] = apn;
            p[u * d + i] = pn;
            part += pn * apn;
        }
    }
    double v[1] = {as_double(part)}, tot[1];
    if (!grid_sum<1>(v, partials, counter, tot)) return;
    if (threadIdx.x == 0)
    {
        ds->pAp = tot[0];
        if (!(tot[0] > 0.0) || !isfinite(tot[0]))
        {
            ds->breakdown = 1;
            ds->done = 1;
            ds->alpha = 0.0;
        }
        else ds->alpha = ds->rz / tot[0];
    }
}

template <int d> struct SpmvGroup { static constexpr int value = d == 3 ? 16 : 8; };

/* The PCG SpMV for d x d blocks: on the sliced-ELL copy of H where there is
   one (thread per block row, coalesced block and column-id loads); else on
   the BSR arrays, a thread per block row for d <= 2 (rows of ~7 2x2 blocks
   on triangle meshes: 41.1 us; the 4- and 8-lane vector form 45.5 / 76.3 us
   on the 1.64M-face disk) and 8 lanes per row for d = 3 (rows of ~15 3x3
   blocks on tet meshes: 27.1 instead of 37.4 us on 663,552 tets). */
template <int d, typename T>
inline void launch_pcg_spmv(cudaStream_t s, const SellView& sv, int64_t nh, const int32_t* bptr, const int32_t* bcol,
                            const T* H, const T* z, T* p, T* Ap, double* partials, unsigned* counter, DevScalars* ds)
{
    if (sv.Hs)
        k_pcg_spmv_sell<d, T><<<PCG_BLOCKS, RED_THREADS, 0, s>>>(nh, sv.sptr, sv.scol, (const T*)sv.Hs, z, p, Ap, partials,
                                                                counter, ds);
    else if constexpr (d == 3)
        k_pcg_spmv_vec<d, T, 8><<<PCG_BLOCKS, RED_THREADS, 0, s>>>(nh, bptr, bcol, H, z, p, Ap, partials, counter, ds);
    else
    {
        // one wave of resident blocks (the grid-stride loop takes the rest)
        static const unsigned grid = std::min<unsigned>(PCG_BLOCKS, resident_grid(k_pcg_spmv_fused<d, T, SpmvGroup<d>::value>,
                                                                                   RED_THREADS));
        k_pcg_spmv_fused<d, T, SpmvGroup<d>::value><<<grid, RED_THREADS, 0, s>>>(nh, bptr, bcol, H, z, p, Ap, partials,
                                                                            counter, ds);
    }
}

template <int d, typename T>
__global__ void __launch_bounds__(RED_THREADS) k_pcg_update(int64_t nh, T* __restrict__ x, T* __restrict__ r, T* __restrict__ z,
                                                            const T* __restrict__ p, const T* __restrict__ Ap,
                                                            const T* __restrict__ dinv, double* partials, unsigned* counter, DevScalars* ds)
{
    if (*(volatile int32_t*)&ds->done) return;
    const T alpha = from_double<T>(ds->alpha);
    T part0 = T(0), part1 = T(0);
    GRID_STRIDE(u, nh)
    {
        // whole block rows per access (8-byte vectors for 2D FP32); x, r, z, p, Ap are distinct buffers
        T xv[d], pv[d], rv[d], av[d], zv[d];
        load_vec<d, T>(x + u * d, xv);
        load_vec<d, T>(p + u * d, pv);
        load_vec<d, T>(r + u * d, rv);
        load_vec<d, T>(Ap + u * d, av);
#pragma unroll
        for (int i = 0; i < d; ++i)
        {
            xv[i] += alpha * pv[i];
            rv[i] -= alpha * av[i];
        }
        store_vec<d, T>(x + u * d, xv);
        store_vec<d, T>(r + u * d, rv);
        apply_dinv<d, T>(dinv, u, rv, zv);
        store_vec<d, T>(z + u * d, zv);
#pragma unroll
        for (int i = 0; i < d; ++i)
        {
            part0 += rv[i] * zv[i];
            part1 += rv[i] * rv[i];
        }
    }
    double v[2] = {as_double(part0), as_double(part1)}, tot[2];
    if (!grid_sum<2>(v, partials, counter, tot)) return;
    if (threadIdx.x == 0)
    {
        ds->beta = tot[0] / ds->rz;
        ds->rz = tot[0];
        ds->rr = tot[1];
        ds->iters += 1;
        if (tot[1] <= ds->tol2 || ds->iters >= ds->max_iters || !isfinite(tot[1])) ds->done = 1;
    }
}

/* ---- vector helpers ------------------------------------------------------ */
__global__ void k_neg(int64_t n, const double* __restrict__ a, double* __restrict__ out)
{
    GRID_STRIDE(i, n) out[i] = -a[i];
}

/* y += x */
__global__ void k_axpy_plain(int64_t n, const double* __restrict__ x, double* __restrict__ y)
{
    GRID_STRIDE(i, n) y[i] += x[i];
}

template <typename T>
__global__ void k_to_double(int64_t n, const T* __restrict__ a, double* __restrict__ out, int accumulate)
{
    // accumulate: 0 = set, 1 = add, -1 = subtract
    GRID_STRIDE(i, n)
    {
        const double v = as_double(a[i]);
        out[i] = accumulate == 0 ? v : out[i] + (accumulate < 0 ? -v : v);
    }
}

/* res = b - (H + wI) y with FP64 accumulation; partial |res|^2 -> ds->rr */
template <int d, typename T>
__global__ void __launch_bounds__(RED_THREADS) k_residual(int64_t nh, const int32_t* __restrict__ bptr, const int32_t* __restrict__ bcol,
                                                          const T* __restrict__ H, double w, const double* __restrict__ y,
                                                          const double* __restrict__ b, double* __restrict__ res,
                                                          double* partials, unsigned* counter, DevScalars* ds)
{
    double part[1] = {0.0};
    GRID_STRIDE(u, nh)
    {
        double acc[d];
#pragma unroll
        for (int i = 0; i < d; ++i) acc[i] = b[u * d + i] - w * y[u * d + i];
        const int32_t b1 = bptr[u + 1];
        for (int32_t bb = bptr[u]; bb < b1; ++bb)
        {
            const int64_t v = bcol[bb];
            const T* B = H + (int64_t)bb * d * d;
#pragma unroll
            for (int i = 0; i < d; ++i)
#pragma unroll
                for (int j = 0; j < d; ++j) acc[i] -= (double)B[i * d + j] * y[v * d + j];
        }
#pragma unroll
        for (int i = 0; i < d; ++i) { res[u * d + i] = acc[i]; part[0] += acc[i] * acc[i]; }
    }
    double tot[1];
    if (!grid_sum<1>(part, partials, counter, tot)) return;
    if (threadIdx.x == 0) ds->rr = tot[0];
}

/* dg = d.g, decrement = -0.5 dg */
__global__ void __launch_bounds__(RED_THREADS) k_dot_dg(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                                                        double* partials, unsigned* counter, DevScalars* ds,
                                                        const int32_t* guard = nullptr)
{
    if (guard && *guard == 0) return;   // guard: a device int, 0 = skip (every block, before the counter)
    double part[1] = {0.0};
    GRID_STRIDE(i, n) part[0] += a[i] * b[i];
    double tot[1];
    if (!grid_sum<1>(part, partials, counter, tot)) return;
    if (threadIdx.x == 0) { ds->dg = tot[0]; ds->decrement = -0.5 * tot[0]; }
}

/* rhs = -g and g.g in one pass (the Newton right-hand side and |g|^2) */
__global__ void __launch_bounds__(RED_THREADS) k_neg_gg(int64_t n, const double* __restrict__ g, double* __restrict__ rhs,
                                                        double* partials, unsigned* counter, DevScalars* ds)
{
    double part[1] = {0.0};
    GRID_STRIDE(i, n)
    {
        const double v = g[i];
        rhs[i] = -v;
        part[0] += v * v;
    }
    double tot[1];
    if (!grid_sum<1>(part, partials, counter, tot)) return;
    if (threadIdx.x == 0) ds->gg = tot[0];
}

/* first trial j (of n) with f_trial[j] <= f + c s_j dg (LineSearch.hh:14-24, :53) */
__global__ void k_ls_select(int n, const double* __restrict__ steps, double c, DevScalars* ds, int adopt = 0,
                            const int32_t* guard = nullptr)
{
    if (threadIdx.x != 0 || blockIdx.x != 0 || (guard && *guard == 0)) return;
    ds->ls_choice = -1;
    for (int j = 0; j < n; ++j)
    {
        const double fn = ds->f_trial[j];
        if (fn != fn) { ds->ls_choice = -2; return; }   // NaN energy
        if (fn <= ds->f + c * steps[j] * ds->dg)
        {
            ds->ls_choice = j;
            ds->ls_f = fn;
            ds->ls_s = steps[j];
            if (adopt) { ds->f_prev = ds->f; ds->f = fn; }   // the accepted point becomes the current one
            return;
        }
    }
}

/* spec_ok = the PCG is done and (diff == NULL or x did not change) */
__global__ void k_spec_guard(DevScalars* ds, const int32_t* diff)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) ds->spec_ok = (ds->done != 0 && (!diff || *diff == 0)) ? 1 : 0;
}

/* *flag = 1 if a and b differ in any bit */
__global__ void k_differs(int64_t n, const double* __restrict__ a, const double* __restrict__ b, int32_t* flag)
{
    bool diff = false;
    GRID_STRIDE(i, n) diff = diff || (__double_as_longlong(a[i]) != __double_as_longlong(b[i]));
    if (__any_sync(0xffffffffu, diff) && (threadIdx.x & 31) == 0) *flag = 1;
}

/* out = a + b */
__global__ void k_add(int64_t n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out,
                      const int32_t* guard = nullptr)
{
    if (guard && *guard == 0) return;
    GRID_STRIDE(i, n) out[i] = a[i] + b[i];
}

/* A mixed solution left in FP32 (d32) to FP64 d, the trial point
   xt = x + d and d.g (with the Newton decrement), in one pass.  The float ->
   double conversions are bit constructions and d.g is accumulated per thread
   in FP32 (the Armijo test scales it by c = 1e-4, so its ~1e-7 relative
   error is immaterial), leaving one FP64 add per entry: the FP64 pipe bound
   this kernel otherwise. */
__global__ void __launch_bounds__(RED_THREADS) k_step_prepare(int64_t n, const float* __restrict__ d32, const double* __restrict__ x,
                                                              const double* __restrict__ g, double* __restrict__ d,
                                                              double* __restrict__ xt, double* partials, unsigned* counter,
                                                              DevScalars* ds, const int32_t* guard)
{
    if (guard && *guard == 0) return;   // every block, before the counter
    float pf = 0.0f;
    GRID_STRIDE(i, n)
    {
        const float vf = d32[i];
        const double v = tad::DoubleFloat::float_to_double(vf);
        d[i] = v;
        xt[i] = x[i] + v;
        pf = fmaf(vf, tad::DoubleFloatValue(g[i]).hi, pf);
    }
    double part[1] = {tad::DoubleFloat::float_to_double(pf)};
    double tot[1];
    if (!grid_sum<1>(part, partials, counter, tot)) return;
    if (threadIdx.x == 0) { ds->dg = tot[0]; ds->decrement = -0.5 * tot[0]; }
}

__global__ void k_axpy_ds(int64_t n, double* __restrict__ x, const double* __restrict__ dx, const DevScalars* ds)
{
    const double s = ds->ls_s;
    GRID_STRIDE(i, n) x[i] += s * dx[i];
}

/* ------------------------------------------------------------------------ */
/* host orchestration                                                        */
/* ------------------------------------------------------------------------ */
static tad_status fail(tad_status s, const std::string& m) { set_error(m); return s; }

/* AMG path, after the V-cycle has produced z: x += alpha p, r -= alpha Ap and
   r.r; the last block counts the iteration and sets the stop flag */
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_pcg_update_nopc(int64_t n, T* x, T* r, const T* __restrict__ p,
                                                                 const T* __restrict__ Ap, double* partials, unsigned* counter,
                                                                 DevScalars* ds)
{
    if (*(volatile int32_t*)&ds->done) return;
    const T alpha = from_double<T>(ds->alpha);
    T part = T(0);
    GRID_STRIDE(i, n)
    {
        x[i] += alpha * p[i];
        const T ri = r[i] - alpha * Ap[i];
        r[i] = ri;
        part += ri * ri;
    }
    double v[1] = {as_double(part)}, tot[1];
    if (!grid_sum<1>(v, partials, counter, tot)) return;
    if (threadIdx.x == 0)
    {
        ds->rr = tot[0];
        ds->iters += 1;
        if (tot[0] <= ds->tol2 || ds->iters >= ds->max_iters || !isfinite(tot[0])) ds->done = 1;
    }
}

/* r.z after the V-cycle: beta = r.z / rz_old, rz = r.z (first: beta = 0) */
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_pcg_rz(int64_t n, const T* __restrict__ r, const T* __restrict__ z,
                                                        double* partials, unsigned* counter, DevScalars* ds, int first)
{
    if (*(volatile int32_t*)&ds->done) return;
    T part = T(0);
    GRID_STRIDE(i, n) part += r[i] * z[i];
    double v[1] = {as_double(part)}, tot[1];
    if (!grid_sum<1>(v, partials, counter, tot)) return;
    if (threadIdx.x == 0)
    {
        if (!(tot[0] > 0.0) || !isfinite(tot[0])) { ds->breakdown = 1; ds->done = 1; return; }
        ds->beta = first ? 0.0 : tot[0] / ds->rz;
        ds->rz = tot[0];
    }
}

constexpr int PCG_CHUNK = 8;   // block-Jacobi iterations per captured graph
constexpr int AMG_CHUNK = 4;   // V-cycle-preconditioned iterations per captured graph

/* The chunk of PCG_CHUNK block-Jacobi iterations as a CUDA graph, captured
   once per (precision, solution buffer, Hessian buffer) and replayed. */
template <int d, typename T>
static tad_status ensure_pcg_graph(Problem& P, T* xs, T* r, T* z, T* p, T* Ap, T* dinv, int prec)
{
    const T* H = (const T*)P.H;
    if (P.pcg_graph && P.pcg_graph_prec == prec && P.pcg_graph_chunk == PCG_CHUNK && P.pcg_graph_x == (const void*)xs &&
        P.pcg_graph_H == (const void*)H)
        return TAD_OK;
    if (P.pcg_graph) { cudaGraphExecDestroy(P.pcg_graph); P.pcg_graph = nullptr; }
    cudaStream_t s = P.stream;
    const int64_t nh = P.n_handles;
    cudaGraph_t graph;
    TAD_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int it = 0; it < PCG_CHUNK; ++it)
    {
        launch_pcg_spmv<d, T>(s, sell_view(P, H), nh, P.bptr, P.bcol, H, z, p, Ap, P.partials, P.counters + 1, P.ds);
        k_pcg_update<d, T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(nh, xs, r, z, p, Ap, dinv, P.partials, P.counters + 2, P.ds);
    }
    TAD_CUDA_TRY(cudaStreamEndCapture(s, &graph));
    TAD_CUDA_TRY(cudaGraphInstantiate(&P.pcg_graph, graph, 0));
    cudaGraphDestroy(graph);
    P.pcg_graph_prec = prec;
    P.pcg_graph_chunk = PCG_CHUNK;
    P.pcg_graph_x = (const void*)xs;
    P.pcg_graph_H = (const void*)H;
    return TAD_OK;
}

/* The chunk of AMG_CHUNK V-cycle-preconditioned CG iterations (fused SpMV,
   then update + V-cycle) as a CUDA graph, captured like ensure_pcg_graph. */
template <int d, typename T>
static tad_status ensure_amg_graph(Problem& P, T* xs, T* r, T* z, T* p, T* Ap, int prec)
{
    const T* H = (const T*)P.H;
    if (P.amg_graph && P.amg_graph_prec == prec && P.amg_graph_x == (const void*)xs && P.amg_graph_H == (const void*)H)
        return TAD_OK;
    tad_status st = amg_build(P);
    if (st != TAD_OK) return st;
    if (P.amg_graph) { cudaGraphExecDestroy(P.amg_graph); P.amg_graph = nullptr; }
    cudaStream_t s = P.stream;
    const int64_t l0 = P.n_launches;
    cudaGraph_t graph;
    TAD_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int it = 0; it < AMG_CHUNK; ++it)
    {
        launch_pcg_spmv<d, T>(s, sell_view(P, H), P.n_handles, P.bptr, P.bcol, H, z, p, Ap, P.partials, P.counters + 1, P.ds);
        P.n_launches += 1;
        amg_apply(P, prec, 1, xs, r, z, p, Ap);
    }
    TAD_CUDA_TRY(cudaStreamEndCapture(s, &graph));
    TAD_CUDA_TRY(cudaGraphInstantiate(&P.amg_graph, graph, 0));
    cudaGraphDestroy(graph);
    P.amg_graph_prec = prec;
    P.amg_graph_x = (const void*)xs;
    P.amg_graph_H = (const void*)H;
    P.amg_graph_launches = P.n_launches - l0;
    P.n_launches = l0;
    return TAD_OK;
}

/* Conjugate gradients preconditioned by one smoothed-aggregation V-cycle
   (amg.cu), restarted from the current iterate (xs, r) of a block-Jacobi
   solve: its tolerance, iteration count and cap carry over. */
template <int d, typename T>
static tad_status pcg_core_amg(Problem& P, T* xs, int* iters_out, T* r, T* z, T* p, T* Ap, int prec)
{
    const int64_t it_switch = P.hs->iters;   // block-Jacobi iterations before the switch
    tad_status st = amg_prepare(P, prec);
    if (st != TAD_OK) return st;
    ++P.amg_solves;
    const T* H = (const T*)P.H;
    const int64_t nh = P.n_handles;
    cudaStream_t s = P.stream;
    amg_apply(P, prec, 0, xs, r, z, p, Ap);
    TAD_CUDA_TRY(cudaGetLastError());
    st = ensure_amg_graph<d, T>(P, xs, r, z, p, Ap, prec);
    if (st != TAD_OK) return st;
    // Replays between host checks: 1, 2, 4, 4, ... chunks -- or, in the
    // Newton loop after a V-cycle solve, first as many chunks as that solve
    // needed, then one at a time.  The iterations a replay runs past
    // convergence return at once but still cost their launches (a V-cycle
    // iteration is a dozen kernels); consecutive hard Newton steps need
    // similar counts.
    const bool predicted = P.in_newton && P.amg_sticky && P.amg_last_chunks > 0;
    int replays = predicted ? std::min(8, P.amg_last_chunks) : 1;
    double rr_last = 0.0;
    int slow = 0;
    for (;;)
    {
        for (int k = 0; k < replays; ++k) TAD_CUDA_TRY(cudaGraphLaunch(P.amg_graph, s));
        P.n_launches += P.amg_graph_launches * replays;
        TAD_CUDA_TRY(cudaMemcpyAsync(P.hs, P.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, s));
        TAD_CUDA_TRY(cudaStreamSynchronize(s));
        if (P.hs->done) break;
        if (sizeof(T) == 4)
        {
            // FP32 V-cycles on a system nearly singular at FP32 rounding
            // level may stop reducing the residual: give up after two host
            // checks without a 10 % reduction (the caller falls back)
            if (rr_last > 0.0 && !(P.hs->rr < 0.9 * rr_last)) ++slow;
            rr_last = P.hs->rr;
            if (slow >= 2)
            {
                if (iters_out) *iters_out = P.hs->iters;
                return TAD_ERR_PCG_NOCONV;
            }
        }
        replays = predicted ? 1 : std::min(4, 2 * replays);
    }
    // the chunks this solve's iterations filled: the next hard solve's first replay
    const int64_t vc_iters = std::max<int64_t>(0, P.hs->iters - it_switch);
    P.amg_last_chunks = P.in_newton ? (int)std::min<int64_t>(8, (vc_iters + AMG_CHUNK - 1) / AMG_CHUNK) : 0;
    if (iters_out) *iters_out = P.hs->iters;
    if (P.hs->breakdown || !(P.hs->rr <= P.hs->tol2)) return TAD_ERR_PCG_NOCONV;
    return TAD_OK;
}

template <int d, typename T>
static tad_status pcg_core(Problem& P, const double* b, T* xs, double w, double rel_tol, int max_iters, int* iters_out,
                           T* r, T* z, T* p, T* Ap, T* dinv, int prec, bool allow_amg = true)
{
    const T* H = (const T*)P.H;
    const int64_t nh = P.n_handles;
    cudaStream_t s = P.stream;
    // P.pcg_async: enqueue init and the first iteration and return PCG_PENDING
    // (the caller checks P.hs->done after its own host round trip);
    // P.pcg_resume: that first iteration ran and P.hs holds its check
    const bool resume = P.pcg_resume;
    P.pcg_resume = false;
    if (!resume)
    {
        k_pcg_init<d, T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(nh, b, xs, r, z, p, Ap, dinv, P.diag, H, w, P.partials, P.counters,
                                                            P.ds, rel_tol, max_iters);
        P.n_launches += 1;
        TAD_CUDA_TRY(cudaGetLastError());
    }
    // The first iteration is launched directly and checked at once (early
    // Newton iterations converge in one); after that, PCG_CHUNK iterations
    // captured once per (precision, solution buffer) are replayed, with the
    // replays between host checks doubling up to 8.  With the AMG policy
    // (preconditioner 1, w = 0: the hierarchy is built from H itself), a
    // solve that has not met its tolerance after the first 1 + PCG_CHUNK
    // iterations continues from its iterate under the smoothed-aggregation
    // V-cycle: block Jacobi has removed the high frequencies by then, and
    // what is left takes it hundreds of iterations on large meshes (the
    // V-cycle: 10-20).  An FP32 solve (mixed precision) whose V-cycles break
    // down or stall falls back to block Jacobi alone, from zero.
    auto launch_iteration = [&]() {
        launch_pcg_spmv<d, T>(s, sell_view(P, H), nh, P.bptr, P.bcol, H, z, p, Ap, P.partials, P.counters + 1, P.ds);
        k_pcg_update<d, T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(nh, xs, r, z, p, Ap, dinv, P.partials, P.counters + 2, P.ds);
    };
    int replays = 0;
    for (;;)
    {
        if (replays == 0)
        {
            if (!resume)
            {
                launch_iteration();
                P.n_launches += 2;
                TAD_CUDA_TRY(cudaGetLastError());
                if (P.pcg_async) return PCG_PENDING;
            }
        }
        else
        {
            const tad_status sg = ensure_pcg_graph<d, T>(P, xs, r, z, p, Ap, dinv, prec);
            if (sg != TAD_OK) return sg;
            for (int k = 0; k < replays; ++k) TAD_CUDA_TRY(cudaGraphLaunch(P.pcg_graph, s));
            P.n_launches += 2 * PCG_CHUNK * replays;
        }
        if (!(resume && replays == 0))
        {
            TAD_CUDA_TRY(cudaMemcpyAsync(P.hs, P.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, s));
            TAD_CUDA_TRY(cudaStreamSynchronize(s));
        }
        if (P.hs->done) { if (allow_amg) P.amg_sticky = false; break; }
        // not done after 1 + PCG_CHUNK iterations -- or after the first, when
        // the previous solve needed the V-cycle: the hard Newton steps of a
        // solve come in a run (the late ones), and each spent PCG_CHUNK
        // block-Jacobi iterations before switching
        const bool slow = replays == 1 || (replays == 0 && P.amg_sticky && P.in_newton);
        // (a problem at or below the coarsest AMG size is one level: its
        // "V-cycle" would be the coarse smoother alone, so block Jacobi goes on)
        if (allow_amg && slow && P.settings.preconditioner == 1 && w == 0.0 && P.amg.size() > 1)
        {
            P.amg_sticky = true;
            // block Jacobi's fast start (the high frequencies) is over and the
            // tolerance is not met: continue from this iterate under the V-cycle
            const tad_status sa = pcg_core_amg<d, T>(P, xs, iters_out, r, z, p, Ap, prec);
            if (sizeof(T) == 8 || sa == TAD_OK) return sa;
            if (P.hs->breakdown == 0 && P.hs->done) return sa;   // the iteration cap
            // FP32: the V-cycle broke down or stalled (a system nearly singular
            // at FP32 rounding level, e.g. the rigid motions of an
            // unconstrained mesh): block Jacobi alone, from zero
            const int used = iters_out ? *iters_out : 0;
            int more = 0;
            const tad_status sj = pcg_core<d, T>(P, b, xs, w, rel_tol, std::max(1, max_iters - used), &more, r, z, p, Ap, dinv,
                                                 prec, false);
            if (iters_out) *iters_out = used + more;
            return sj;
        }
        replays = replays == 0 ? 1 : std::min(8, 2 * replays);
    }
    if (iters_out) *iters_out = P.hs->iters;
    if (P.hs->breakdown) return TAD_ERR_PCG_NOCONV;
    if (!(P.hs->rr <= P.hs->tol2)) return TAD_ERR_PCG_NOCONV;
    return TAD_OK;
}

/* FP64 solve of H64 e = res on the FP64 copy of the FP32 Hessian, added to
   xsol (the robust completion of a tight mixed-precision solve) */
template <int d>
static tad_status mixed_fp64_completion(Problem& P, const double* res, double* xsol, double rel_tol, int max_iters, int* iters)
{
    cudaStream_t s = P.stream;
    const int64_t nv = P.nb * d * d;
    if (!P.Hd) TAD_CUDA_TRY(cudaMalloc(&P.Hd, std::max<int64_t>(nv, 1) * sizeof(double)));
    k_to_double<float><<<RED_BLOCKS, RED_THREADS, 0, s>>>(nv, (const float*)P.H, (double*)P.Hd, 0);
    P.n_launches += 1;
    if (!P.corr) TAD_CUDA_TRY(cudaMalloc(&P.corr, std::max<int64_t>(P.n_vars, 1) * sizeof(double)));
    void* keep = P.H;
    P.H = P.Hd;
    int it = 0;
    // the correction goes to its own buffer: xsol may be P.dx
    const tad_status st = pcg_core<d, double>(P, res, P.corr, 0.0, rel_tol, max_iters, &it, P.r, P.z, P.p, P.Ap, P.dinv, 0);
    P.H = keep;
    *iters += it;
    k_axpy_plain<<<RED_BLOCKS, RED_THREADS, 0, s>>>(P.n_vars, P.corr, xsol);
    P.n_launches += 1;
    return st;
}

template <int d>
static tad_status pcg_dispatch(Problem& P, const double* b, double* xsol, int precision, double rel_tol, int max_iters, int* iters)
{
    const int64_t n = P.n_vars;
    cudaStream_t s = P.stream;
    if (precision != TAD_PREC_MIXED)
        return pcg_core<d, double>(P, b, xsol, 0.0, rel_tol, max_iters, iters, P.r, P.z, P.p, P.Ap, P.dinv, 0);
    // mixed: FP64 iterative refinement around FP32 PCG.  The first pass
    // solves H dx = b from dx = 0 (its init kernel also returns |b|^2 in
    // FP64).  For a loose tolerance (>= LOOSE_TOL) the FP32 solve meets the
    // tolerance by itself -- its recursively updated residual drifts from the
    // true one by O(eps_fp32 cond(H)) relative, far below 1e-4 -- so that pass
    // is the answer; tighter tolerances compute r = b - H x in FP64 and solve
    // for corrections until the FP64 residual meets them.  FP32 CG on a nearly
    // singular H (the eps-regularised rigid motions of an unconstrained mesh)
    // stalls or diverges at tight tolerances: a pass that increases the FP64
    // residual is undone, and once a pass reduces its norm by less than
    // MIN_PASS_GAIN (or the passes run out) the rest is solved in FP64 on an
    // FP64 copy of the FP32 Hessian (same matrix, so the result is still exact
    // to the FP32-evaluated Hessian).
    constexpr double LOOSE_TOL = MIXED_LOOSE_TOL;
    constexpr double MIN_PASS_GAIN = 100.0;
    const double tol = P.settings.refine_rel_tol;
    const double inner_tol = std::max(rel_tol, 1e-6);
    int total = 0;
    tad_status st = pcg_core<d, float>(P, b, P.dx32, 0.0, inner_tol, max_iters, &total, P.r32, P.z32, P.p32, P.Ap32, P.dinv32, 1);
    if (st == PCG_PENDING) return st;   // async first iteration (loose tolerances only)
    const double bb = P.hs->bb;
    if (rel_tol >= LOOSE_TOL || bb == 0.0)
    {
        if (P.defer_fp32 && xsol == P.dx) P.solution_in_dx32 = true;   // the caller converts it (k_step_prepare)
        else
        {
            k_to_double<float><<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, P.dx32, xsol, 0);
            P.n_launches += 1;
        }
        if (iters) *iters = total;
        return st;
    }
    k_to_double<float><<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, P.dx32, xsol, 0);
    P.n_launches += 1;
    const double target = std::min(rel_tol, std::max(tol, 0.0));
    double rr_prev = bb;
    bool completion = false;
    const int passes = std::max(1, P.settings.refine_max_iters);
    for (int pass = 0;; ++pass)
    {
        k_residual<d, float><<<RED_BLOCKS, RED_THREADS, 0, s>>>(P.n_handles, P.bptr, P.bcol, (const float*)P.H, 0.0, xsol, b, P.res,
                                                                P.partials, P.counters + 3, P.ds);
        P.n_launches += 1;
        TAD_CUDA_TRY(cudaMemcpyAsync(P.hs, P.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, s));
        TAD_CUDA_TRY(cudaStreamSynchronize(s));
        const double rr = P.hs->rr;
        if (rr <= target * target * bb || total >= max_iters) break;
        if (!(rr < rr_prev))
        {
            // the last FP32 pass made the residual worse: undo it, finish in FP64
            k_to_double<float><<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, P.dx32, xsol, -1);
            k_residual<d, float><<<RED_BLOCKS, RED_THREADS, 0, s>>>(P.n_handles, P.bptr, P.bcol, (const float*)P.H, 0.0, xsol, b,
                                                                    P.res, P.partials, P.counters + 3, P.ds);
            P.n_launches += 2;
            completion = true;
            break;
        }
        if (!(rr <= rr_prev / (MIN_PASS_GAIN * MIN_PASS_GAIN)) || pass + 1 >= passes)
        {
            // FP32 passes are not effective here (or none are left): keep this
            // one, finish in FP64 from the residual just computed
            completion = true;
            break;
        }
        rr_prev = rr;
        int it = 0;
        st = pcg_core<d, float>(P, P.res, P.dx32, 0.0, inner_tol, max_iters - total, &it, P.r32, P.z32, P.p32, P.Ap32, P.dinv32, 1);
        total += it;
        k_to_double<float><<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, P.dx32, xsol, 1);
        P.n_launches += 1;
    }
    if (completion)
    {
        // res holds b - H x for the current x; relative target against |b|
        TAD_CUDA_TRY(cudaMemcpyAsync(P.hs, P.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, s));
        TAD_CUDA_TRY(cudaStreamSynchronize(s));
        const double rres = std::sqrt(std::max(P.hs->rr, 0.0));
        const double rel = rres > 0.0 ? std::min(0.5, target * std::sqrt(bb) / rres) : 0.5;
        st = mixed_fp64_completion<d>(P, P.res, xsol, rel, std::max(1, max_iters - total), &total);
        k_residual<d, float><<<RED_BLOCKS, RED_THREADS, 0, s>>>(P.n_handles, P.bptr, P.bcol, (const float*)P.H, 0.0, xsol, b, P.res,
                                                                P.partials, P.counters + 3, P.ds);
        P.n_launches += 1;
        TAD_CUDA_TRY(cudaMemcpyAsync(P.hs, P.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, s));
        TAD_CUDA_TRY(cudaStreamSynchronize(s));
    }
    if (iters) *iters = total;
    if (!(P.hs->rr <= rel_tol * rel_tol * bb * 1.0001) && !(P.hs->rr <= tol * tol * bb)) return TAD_ERR_PCG_NOCONV;
    return st == TAD_ERR_PCG_NOCONV ? TAD_OK : st;
}

/* The captured iteration graphs of the Newton loop's solves (its solution and
   vector buffers, the problem's precision), at finalisation, so that the
   first solve needing them does not capture them */
template <int d>
static tad_status prepare_graphs_d(Problem& P)
{
    const bool amg = P.settings.preconditioner == 1 && P.amg.size() > 1;
    if (P.precision == TAD_PREC_MIXED)
    {
        tad_status st = ensure_pcg_graph<d, float>(P, P.dx32, P.r32, P.z32, P.p32, P.Ap32, P.dinv32, 1);
        if (st == TAD_OK && amg) st = ensure_amg_graph<d, float>(P, P.dx32, P.r32, P.z32, P.p32, P.Ap32, 1);
        return st;
    }
    tad_status st = ensure_pcg_graph<d, double>(P, P.dx, P.r, P.z, P.p, P.Ap, P.dinv, 0);
    if (st == TAD_OK && amg) st = ensure_amg_graph<d, double>(P, P.dx, P.r, P.z, P.p, P.Ap, 0);
    return st;
}

tad_status prepare_solver_graphs(Problem& P)
{
    switch (P.d)
    {
    case 1: return prepare_graphs_d<1>(P);
    case 2: return prepare_graphs_d<2>(P);
    default: return prepare_graphs_d<3>(P);
    }
}

/* H += w I on the assembled diagonal blocks */
template <int d, typename T>
__global__ void k_add_diag(int64_t nh, const int32_t* __restrict__ diag, T* __restrict__ H, double w,
                           const int32_t* __restrict__ sdiag, T* __restrict__ Hs)
{
    GRID_STRIDE(u, nh)
    {
        const int32_t b = diag[u];
        if (b < 0) continue;
#pragma unroll
        for (int i = 0; i < d; ++i) H[(int64_t)b * d * d + i * d + i] += (T)w;
        if (Hs)
#pragma unroll
            for (int i = 0; i < d; ++i) Hs[(int64_t)sdiag[u] * d * d + i * d + i] += (T)w;   // the sliced-ELL copy too
    }
}

void add_identity(Problem& P, double w, int precision)
{
    const bool fp32 = precision == TAD_PREC_MIXED;
    switch (P.d)
    {
    case 1: fp32 ? k_add_diag<1, float><<<RED_BLOCKS, RED_THREADS, 0, P.stream>>>(P.n_handles, P.diag, (float*)P.H, w, P.sdiag, (float*)P.Hs)
                 : k_add_diag<1, double><<<RED_BLOCKS, RED_THREADS, 0, P.stream>>>(P.n_handles, P.diag, (double*)P.H, w, P.sdiag, (double*)P.Hs); break;
    case 2: fp32 ? k_add_diag<2, float><<<RED_BLOCKS, RED_THREADS, 0, P.stream>>>(P.n_handles, P.diag, (float*)P.H, w, P.sdiag, (float*)P.Hs)
                 : k_add_diag<2, double><<<RED_BLOCKS, RED_THREADS, 0, P.stream>>>(P.n_handles, P.diag, (double*)P.H, w, P.sdiag, (double*)P.Hs); break;
    default: fp32 ? k_add_diag<3, float><<<RED_BLOCKS, RED_THREADS, 0, P.stream>>>(P.n_handles, P.diag, (float*)P.H, w, P.sdiag, (float*)P.Hs)
                  : k_add_diag<3, double><<<RED_BLOCKS, RED_THREADS, 0, P.stream>>>(P.n_handles, P.diag, (double*)P.H, w, P.sdiag, (double*)P.Hs); break;
    }
    P.n_launches += 1;
}

tad_status pcg_solve(Problem& P, const double* b, double* xsol, double w_identity, int precision, double rel_tol,
                     int max_iters, int* iters_out)
{
    if (w_identity != 0.0) return fail(TAD_ERR_ARG, "w_identity must be 0 on the device path");
    switch (P.d)
    {
    case 1: return pcg_dispatch<1>(P, b, xsol, precision, rel_tol, max_iters, iters_out);
    case 2: return pcg_dispatch<2>(P, b, xsol, precision, rel_tol, max_iters, iters_out);
    default: return pcg_dispatch<3>(P, b, xsol, precision, rel_tol, max_iters, iters_out);
    }
}

/* reference step sequence (LineSearch.hh:41-59) */
static void step_sequence(double s_max, double shrink, int n, std::vector<double>& out)
{
    const bool try_one = s_max > 1.0;
    double s = s_max;
    out.resize(n);
    for (int i = 0; i < n; ++i)
    {
        out[i] = s;
        if (try_one && s > 1.0 && s * shrink < 1.0) s = 1.0;
        else s *= shrink;
    }
}

/* The step sequence for (s_max, shrink, n) in P.steps_seq, uploaded only
   when the key changes. */
static tad_status ensure_step_sequence(Problem& P, double s_max, int n)
{
    const double shrink = P.settings.ls_shrink;
    if (P.steps_seq && P.steps_key[0] == s_max && P.steps_key[1] == shrink && P.steps_key[2] == (double)n) return TAD_OK;
    if (n > P.steps_seq_cap)
    {
        if (P.steps_seq) TAD_CUDA_TRY(cudaFree(P.steps_seq));
        P.steps_seq = nullptr;
        TAD_CUDA_TRY(cudaMalloc(&P.steps_seq, (size_t)n * sizeof(double)));
        P.steps_seq_cap = n;
    }
    std::vector<double> seq;
    step_sequence(s_max, shrink, n, seq);
    TAD_CUDA_TRY(cudaMemcpyAsync(P.steps_seq, seq.data(), (size_t)n * sizeof(double), cudaMemcpyHostToDevice, P.stream));
    TAD_CUDA_TRY(cudaStreamSynchronize(P.stream));   // seq is a host temporary
    P.steps_key[0] = s_max; P.steps_key[1] = shrink; P.steps_key[2] = (double)n;
    return TAD_OK;
}

tad_status line_search_device(Problem& P, double* x, const double* d, double f, double s_max, bool* found,
                              double* f_out, int* trials, bool f_on_device, int t_start, double stop_decrement,
                              bool* stopped)
{
    if (stopped) *stopped = false;
    cudaStream_t s = P.stream;
    const int max_iters = P.settings.ls_max_iters > 0 ? P.settings.ls_max_iters : 64;
    tad_status st = ensure_step_sequence(P, s_max, max_iters);
    if (st != TAD_OK) return st;
    if (t_start == 0)
    {
        k_dot_dg<<<RED_BLOCKS, RED_THREADS, 0, s>>>(P.n_vars, d, P.g, P.partials, P.counters + 4, P.ds);
        P.n_launches += 1;
    }
    // current energy: ds->f, from the caller unless it is already there
    if (!f_on_device) TAD_CUDA_TRY(cudaMemcpyAsync(&P.ds->f, &f, sizeof(double), cudaMemcpyHostToDevice, s));
    *found = false;
    int t0 = t_start;
    int batch = t_start == 0 ? 1 : LS_BATCH;
    while (t0 < max_iters)
    {
        const int nb = std::min(batch, max_iters - t0);
        double* keep = P.steps;
        P.steps = P.steps_seq + t0;
        st = eval_elements(P, TAD_MODE_LINESEARCH, x, 0.0, P.precision, d, nb);
        P.steps = keep;
        if (st != TAD_OK) return st;
        launch_reduce_f(P, nb, P.ds->f_trial);
        k_ls_select<<<1, 32, 0, s>>>(nb, P.steps_seq + t0, P.settings.ls_armijo, P.ds);
        P.n_launches += 2;
        TAD_CUDA_TRY(cudaMemcpyAsync(P.hs, P.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, s));
        TAD_CUDA_TRY(cudaMemcpyAsync(P.err_h, P.err, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        TAD_CUDA_TRY(cudaStreamSynchronize(s));
        // an element error of this step (or of the evaluation before it) first
        if (*P.err_h != 0) return check_device_error(P);
        if (stop_decrement > 0.0 && P.hs->decrement < stop_decrement)
        {
            // converged by the Newton decrement: no step (the reference tests it before line_search)
            if (stopped) *stopped = true;
            if (f_out) *f_out = f_on_device ? P.hs->f : f;
            if (trials) *trials = 0;
            return TAD_OK;
        }
        if (P.hs->ls_choice == -2) return fail(TAD_ERR_NONFINITE, "Assertion failed: f_new == f_new (NaN energy in line search)");
        if (P.hs->ls_choice >= 0)
        {
            k_axpy_ds<<<RED_BLOCKS, RED_THREADS, 0, s>>>(P.n_vars, x, d, P.ds);
            P.n_launches += 1;
            *found = true;
            if (f_out) *f_out = P.hs->ls_f;
            if (trials) *trials = t0 + P.hs->ls_choice + 1;
            return TAD_OK;
        }
        t0 += nb;
        batch = LS_BATCH;
    }
    if (f_out) *f_out = f_on_device ? P.hs->f : f;
    if (trials) *trials = max_iters;
    return TAD_OK;
}

/* The first line-search trial (s = 1) evaluated as the next iteration's
   derivatives: x_t = x + d, the full element kernels and assembly at x_t,
   the trial energy into f_trial[0] and the Armijo test (which makes it the
   current energy if it passes).  Returns the selection in P.hs after one
   host round trip; the caller adopts x_t (its derivatives are then already
   assembled) or continues the line search at trial 2. */
static tad_status speculative_first_trial(Problem& P, const double* x, double* d, double* xt, double eps, bool d_in_fp32,
                                         const int32_t* guard = nullptr, double* out_h = nullptr)
{
    // out_h: xt is copied to this host buffer on the side stream as soon as it
    // is formed, beside the element kernels (ordered after any earlier copy)
    // guard (the PCG's done flag): every kernel here returns at once while it
    // is 0, so the block can be enqueued behind an unchecked PCG iteration
    cudaStream_t s = P.stream;
    if (d_in_fp32)
    {
        k_step_prepare<<<RED_BLOCKS, RED_THREADS, 0, s>>>(P.n_vars, P.dx32, x, P.g, d, xt, P.partials, P.counters + 4, P.ds, guard);
        P.n_launches += 1;
    }
    else
    {
        k_dot_dg<<<RED_BLOCKS, RED_THREADS, 0, s>>>(P.n_vars, d, P.g, P.partials, P.counters + 4, P.ds, guard);
        k_add<<<RED_BLOCKS, RED_THREADS, 0, s>>>(P.n_vars, x, d, xt, guard);
        P.n_launches += 2;
    }
    if (out_h)
    {
        cudaEventRecord(P.ev_xt, s);   // xt is final from here on
        cudaStreamWaitEvent(P.stream2, P.ev_xt, 0);
        cudaMemcpyAsync(out_h, xt, P.n_vars * sizeof(double), cudaMemcpyDeviceToHost, P.stream2);
        cudaEventRecord(P.ev_out, P.stream2);
    }
    P.launch_guard = guard;
    tad_status st = eval_elements(P, TAD_MODE_HESSIAN_PROJ, xt, eps, P.precision);
    if (st == TAD_OK) st = assemble(P, true, true, P.precision, P.ds->f_trial, true);
    P.launch_guard = nullptr;
    if (st != TAD_OK) return st;
    k_ls_select<<<1, 32, 0, s>>>(1, P.steps_seq, P.settings.ls_armijo, P.ds, 1, guard);
    P.n_launches += 1;
    TAD_CUDA_TRY(cudaMemcpyAsync(P.hs, P.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, s));
    TAD_CUDA_TRY(cudaMemcpyAsync(P.err_h, P.err, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    TAD_CUDA_TRY(cudaStreamSynchronize(s));
    return TAD_OK;
}

tad_status newton_solve(Problem& P, double* x, int n_iters, double eps, double stop_decrement, double* f_hist, int* iters_done,
                        const double* x_in_h, double* x_out_h)
{
    tad_status s = ensure_finalized(P);
    if (s != TAD_OK) return s;
    cudaStream_t st = P.stream;
    const int prec = P.precision;
    for (int i = 0; i < 4; ++i) P.ms_stage[i] = 0.0;
    P.pcg_iters_total = 0;
    P.ls_trials_total = 0;
    // Without the forcing sequence nothing on the host needs f or |g| before
    // the line search, so the iteration runs without a host round trip until
    // the PCG's first check: f stays in ds->f, and the element error word is
    // read with the line search's scalars (an element error there stops the
    // iteration before x is updated).
    //
    // The full step s = 1 is tried first and is accepted in almost every
    // iteration of a Newton solve; its energy is then evaluated by the full
    // element kernels at x + d, which are the next iteration's derivatives
    // (speculative_first_trial).  A rejection falls back to the energy-only
    // line search from trial 2, with the same trial sequence and Armijo test,
    // and turns the speculation off until a full step is accepted again.  The
    // accepted state alternates between x and P.x_trial; x holds it on return.
    //
    // Across calls: a call that starts from the exact x the previous call
    // returned (a bitwise device compare) continues that solve.  Once calls
    // have continued each other twice in a row, the last iteration of a call
    // speculates too, and the next continuing call starts from the
    // derivatives it assembled (as an iteration inside one call would),
    // provided nothing else has evaluated on the problem since and eps and
    // precision are the same.  Such a call is predicted to continue: its
    // PCG starts on the carried derivatives while x is copied in and
    // compared on the side stream, and the speculative block waits for the
    // compare and runs only if x is unchanged; a call whose x changed reruns
    // its first iteration from an evaluation.  A one-iteration call copies
    // its result out on the side stream as soon as the trial point x + d is
    // formed, beside the speculative evaluation.
    const bool forcing = P.settings.forcing == 1;
    const int ls_max = P.settings.ls_max_iters > 0 ? P.settings.ls_max_iters : 64;
    const int64_t n = P.n_vars;
    cudaStream_t st2 = P.stream2;
    if (!P.x_trial) TAD_CUDA_TRY(cudaMalloc(&P.x_trial, std::max<int64_t>(n, 1) * sizeof(double)));
    if (!P.last_x) TAD_CUDA_TRY(cudaMalloc(&P.last_x, std::max<int64_t>(n, 1) * sizeof(double)));
    if (!P.diff_flag) TAD_CUDA_TRY(cudaMalloc(&P.diff_flag, sizeof(int32_t)));
    if (!P.diff_flag_h) TAD_CUDA_TRY(cudaMallocHost(&P.diff_flag_h, sizeof(int32_t)));
    s = ensure_step_sequence(P, 1.0, ls_max);
    if (s != TAD_OK) return s;
    // input copy and continuation test on the side stream (ordered after the
    // main stream's earlier work on x)
    const bool predicted = P.last_x_valid && P.spec_valid && P.spec_eps == eps && P.spec_prec == prec;
    P.spec_valid = false;
    TAD_CUDA_TRY(cudaEventRecord(P.ev_in, st));
    // A predicted call issues the side-stream work after its PCG's first
    // launches (the PCG does not read x), so the GPU starts on the PCG
    // without waiting for these API calls; the copy still waits only for the
    // work recorded above.
    bool input_issued = false;
    auto issue_input = [&]() -> cudaError_t {
        input_issued = true;
        cudaError_t e = cudaStreamWaitEvent(st2, P.ev_in, 0);
        if (e == cudaSuccess && x_in_h) e = cudaMemcpyAsync(x, x_in_h, n * sizeof(double), cudaMemcpyHostToDevice, st2);
        if (e == cudaSuccess) e = cudaMemsetAsync(P.diff_flag, 0, sizeof(int32_t), st2);
        if (e == cudaSuccess && P.last_x_valid)
        {
            k_differs<<<RED_BLOCKS, RED_THREADS, 0, st2>>>(n, x, P.last_x, P.diff_flag);
            P.n_launches += 1;
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(P.ev_in, st2);
        return e;
    };
    if (!predicted) TAD_CUDA_TRY(issue_input());
    bool continues = false;
    bool pending_test = predicted;   // the continuation test is read after iteration 0's first sync
    if (!predicted)
    {
        TAD_CUDA_TRY(cudaStreamWaitEvent(st, P.ev_in, 0));   // the evaluation reads x
        if (P.last_x_valid)
        {
            TAD_CUDA_TRY(cudaMemcpyAsync(P.diff_flag_h, P.diff_flag, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
            TAD_CUDA_TRY(cudaStreamSynchronize(st));
            continues = *P.diff_flag_h == 0;
        }
        P.streak = continues ? P.streak + 1 : 0;
        if (!continues) P.amg_sticky = false;   // a new solve: its PCG history starts here
    }
    double* cur = x;
    double* spare = P.x_trial;
    bool have_derivs = predicted;   // derivatives at cur already assembled (accepted speculative step)
    bool early_out = false;         // a copy of spare to x_out_h was issued on the side stream
    double* early_buf = nullptr;
    struct NewtonScope
    {
        Problem& P;
        ~NewtonScope() { P.in_newton = false; }
    } newton_scope{P};
    P.in_newton = true;
    auto finish = [&](tad_status rs) {
        if (!input_issued)
        {
            // a predicted call that stopped before its first PCG (no iteration
            // asked for, or an error): x takes the input before it is used
            // below; a failed copy is the call's status (x may be stale)
            const cudaError_t e = issue_input();
            if (e == cudaSuccess) cudaStreamWaitEvent(st, P.ev_in, 0);
            else if (rs == TAD_OK)
            {
                set_error(std::string("CUDA error: ") + cudaGetErrorString(e) + " (input copy)");
                rs = TAD_ERR_CUDA;
            }
        }
        if (cur != x) cudaMemcpyAsync(x, cur, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
        const bool ok = rs == TAD_OK;
        if (ok) cudaMemcpyAsync(P.last_x, x, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
        if (x_out_h)
        {
            // the early copy holds the result when it was taken of the accepted
            // trial point; otherwise (after it, if any) copy x out -- on an
            // error x still holds the call's input (one-iteration calls)
            const bool early_good = ok && early_out && early_buf == cur && have_derivs;
            if (!early_good && (ok || early_out))
            {
                if (early_out) cudaStreamWaitEvent(st, P.ev_out, 0);
                cudaMemcpyAsync(x_out_h, x, n * sizeof(double), cudaMemcpyDeviceToHost, st);
            }
        }
        cudaStreamSynchronize(st);
        cudaStreamSynchronize(st2);
        P.last_x_valid = ok;
        // carried derivatives stay valid only if this call's continuation
        // test was read (a predicted call with no iteration never reads it)
        P.spec_valid = ok && have_derivs && !pending_test;
        P.spec_eps = eps;
        P.spec_prec = prec;
        return rs;
    };
    if (P.stage_ev.empty())
    {
        P.stage_ev.resize(5 * Problem::STAGE_ITERS, nullptr);
        for (auto& e : P.stage_ev) TAD_CUDA_TRY(cudaEventCreate(&e));
    }
    auto ev = [&](int i, int k) { return P.stage_ev[5 * std::min(i, Problem::STAGE_ITERS - 1) + k]; };
    bool speculate = true;
    bool all_builtin = true;
    for (const Term& T : P.terms) all_builtin = all_builtin && T.energy >= 0;
    double f = 0.0;
    int it = 0;
    for (; it < n_iters; ++it)
    {
        cudaEventRecord(ev(it, 0), st);
        if (!have_derivs)
        {
            s = eval_elements(P, TAD_MODE_HESSIAN_PROJ, cur, eps, prec);
            if (s != TAD_OK) return finish(s);
        }
        cudaEventRecord(ev(it, 1), st);
        if (!have_derivs)
        {
            // f, g, H, and rhs = -g with |g|^2 (an accepted speculative step assembled them already)
            s = assemble(P, true, true, prec, nullptr, true);
            if (s != TAD_OK) return finish(s);
        }
        cudaEventRecord(ev(it, 2), st);
        double tol = P.settings.pcg_rel_tol;
        if (forcing)
        {
            s = check_device_error(P);
            if (s != TAD_OK) return finish(s);
            TAD_CUDA_TRY(cudaMemcpyAsync(P.hs, P.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
            TAD_CUDA_TRY(cudaStreamSynchronize(st));
            const double gnorm = std::sqrt(P.hs->gg);
            if (P.g0_norm == 0.0) P.g0_norm = gnorm;   // first iteration since create / set_settings
            if (P.g0_norm > 0.0) tol = std::max(tol, std::min(0.5, std::sqrt(gnorm / P.g0_norm)));
        }
        // the last iteration speculates only once calls have continued each
        // other twice in a row (a caller stepping a solve call by call)
        const int streak_now = pending_test ? P.streak + 1 : P.streak;   // a predicted call continues
        const bool spec_now = speculate && (it + 1 < n_iters || streak_now >= 2);
        // one-iteration calls with a host output copy it out early (beside the speculative evaluation)
        double* const out_early = (x_out_h && n_iters == 1 && spec_now) ? x_out_h : nullptr;
        // The speculative trial is enqueued right behind the PCG's first
        // iteration, guarded by its done flag, so that one host round trip
        // serves both when the first iteration converges (it does in most
        // iterations of a solve).  Only for one-pass solves (FP64, or mixed at
        // a loose tolerance) and built-in energies, whose kernels honour the
        // guard.
        const bool async = spec_now && !forcing && all_builtin && (prec != TAD_PREC_MIXED || tol >= MIXED_LOOSE_TOL);
        int pit = 0;
        P.defer_fp32 = spec_now;
        P.solution_in_dx32 = false;
        P.pcg_async = async;
        s = pcg_solve(P, P.rhs, P.dx, 0.0, prec, tol, P.settings.pcg_max_iters, &pit);
        P.pcg_async = false;
        if (!input_issued) TAD_CUDA_TRY(issue_input());
        bool trial_done = false;
        bool d_in_fp32 = P.solution_in_dx32;
        // the speculative block of a predicted call's first iteration waits for
        // the input copy and the continuation test, and runs only if x is the
        // state the carried derivatives belong to
        auto spec_guard = [&](const int32_t* pcg_done) -> const int32_t* {
            if (!pending_test) return pcg_done;
            cudaStreamWaitEvent(st, P.ev_in, 0);   // errors surface at the next checked call
            k_spec_guard<<<1, 32, 0, st>>>(P.ds, P.last_x_valid ? P.diff_flag : nullptr);
            cudaMemcpyAsync(P.diff_flag_h, P.diff_flag, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
            P.n_launches += 1;
            return &P.ds->spec_ok;
        };
        auto launch_early_out = [&]() {
            if (!out_early) return;
            early_out = true;   // speculative_first_trial issued the copy of spare
            early_buf = spare;
        };
        bool spec_issued = false;
        if (s == PCG_PENDING)
        {
            // a loose mixed solve leaves its solution in dx32, FP64 in P.dx
            d_in_fp32 = prec == TAD_PREC_MIXED;
            s = speculative_first_trial(P, cur, P.dx, spare, eps, d_in_fp32, spec_guard(&P.ds->done), out_early);
            launch_early_out();
            spec_issued = true;
            if (s != TAD_OK) return finish(s);
            if (P.hs->done)
            {
                trial_done = true;
                pit = P.hs->iters;
                s = (P.hs->breakdown || !(P.hs->rr <= P.hs->tol2)) ? TAD_ERR_PCG_NOCONV : TAD_OK;
            }
            else
            {
                // not converged in one iteration: the guarded block did nothing
                P.pcg_resume = true;
                P.solution_in_dx32 = false;
                s = pcg_solve(P, P.rhs, P.dx, 0.0, prec, tol, P.settings.pcg_max_iters, &pit);
                P.pcg_resume = false;
                d_in_fp32 = P.solution_in_dx32;
            }
        }
        P.defer_fp32 = false;
        P.solution_in_dx32 = false;
        P.pcg_iters_total += pit;
        if (s != TAD_OK && s != TAD_ERR_PCG_NOCONV) return finish(s);
        cudaEventRecord(ev(it, 3), st);
        bool found = false;
        bool stopped = false;   // the Newton decrement fell below stop_decrement: no step
        double fn = 0.0;
        int trials = 0;
        have_derivs = false;
        if (spec_now && !trial_done)
        {
            // The PCG was checked on the host (not pending, or resumed after a
            // guarded block that ran without effect).  A predicted call whose
            // test result is already known runs the trial unguarded, unless x
            // changed (the iteration then reruns, below); one whose test is
            // still on the side stream guards the trial with it.
            const bool test_known = pending_test && spec_issued;
            if (!(test_known && *P.diff_flag_h != 0))
            {
                const int32_t* g = (pending_test && !test_known) ? spec_guard(&P.ds->done) : nullptr;
                const tad_status s2 = speculative_first_trial(P, cur, P.dx, spare, eps, d_in_fp32, g, out_early);
                if (s2 != TAD_OK) return finish(s2);
                launch_early_out();
            }
        }
        if (pending_test)
        {
            // the continuation test (copied with the first host round trip; a
            // first iteration that did not speculate reads it here)
            if (!spec_now)
            {
                TAD_CUDA_TRY(cudaStreamWaitEvent(st, P.ev_in, 0));
                TAD_CUDA_TRY(cudaMemcpyAsync(P.diff_flag_h, P.diff_flag, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
                TAD_CUDA_TRY(cudaStreamSynchronize(st));
            }
            pending_test = false;
            continues = *P.diff_flag_h == 0;
            if (!continues)
            {
                // x changed: everything above used derivatives of another state
                P.streak = 0;
                P.amg_sticky = false;   // a new solve: its PCG history starts here
                have_derivs = false;
                speculate = true;
                --it;
                continue;
            }
            P.streak = P.streak + 1;
        }
        if (spec_now)
        {
            if (s != TAD_OK && s != TAD_ERR_PCG_NOCONV) return finish(s);
            const int choice = P.hs->ls_choice;
            if (stop_decrement > 0.0 && P.hs->decrement < stop_decrement)
            {
                // converged by the Newton decrement (d.g was reduced before the
                // selection): the reference stops before line_search, so x keeps
                // this iteration's start; the trial's derivatives and any error
                // it reported are dropped
                stopped = true;
                if (*P.err_h != 0) TAD_CUDA_TRY(cudaMemsetAsync(P.err, 0, sizeof(int32_t), st));
                fn = choice == 0 ? P.hs->f_prev : P.hs->f;   // an accepted trial moved ds->f on
            }
            else if (choice == -2)
                return finish(fail(TAD_ERR_NONFINITE, "Assertion failed: f_new == f_new (NaN energy in line search)"));
            else if (choice == 0)
            {
                // accepted: x + d is the new state, its derivatives are assembled
                std::swap(cur, spare);
                have_derivs = true;
                found = true;
                fn = P.hs->ls_f;
                trials = 1;
                if (*P.err_h != 0) return finish(check_device_error(P));   // as the next evaluation would report
            }
            else
            {
                // rejected: derivatives at x + d are not needed (clear what they reported)
                if (*P.err_h != 0) TAD_CUDA_TRY(cudaMemsetAsync(P.err, 0, sizeof(int32_t), st));
                s = line_search_device(P, cur, P.dx, 0.0, 1.0, &found, &fn, &trials, true, 1);
                if (s != TAD_OK) return finish(s);
                speculate = false;
            }
        }
        else
        {
            s = line_search_device(P, cur, P.dx, 0.0, 1.0, &found, &fn, &trials, true, 0, stop_decrement, &stopped);
            if (s != TAD_OK) return finish(s);
            speculate = found && trials == 1;
        }
        cudaEventRecord(ev(it, 4), st);
        if (stopped)
        {
            // iterations done = steps taken; f_hist[it] is the final energy
            f = fn;
            break;
        }
        // the energy at the start of this iteration (ds->f, or what an accepted
        // speculative step replaced there)
        f = have_derivs ? P.hs->f_prev : P.hs->f;
        if (f_hist) f_hist[it] = f;
        P.ls_trials_total += trials;
        f = fn;
        if (!found) { ++it; break; }
    }
    if (f_hist) f_hist[it] = f;
    if (iters_done) *iters_done = it;
    const tad_status rs = finish(TAD_OK);   // synchronises the stream
    // stage times, from the events the iterations recorded (the last slot is
    // shared by iterations beyond STAGE_ITERS - 1, which are not counted)
    for (int i = 0; i < std::min(it, Problem::STAGE_ITERS - 1); ++i)
        for (int k = 0; k < 4; ++k)
        {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, ev(i, k), ev(i, k + 1)) == cudaSuccess) P.ms_stage[k] += ms;
        }
    cudaGetLastError();
    return rs;
}

} // namespace tadlib

using namespace tadlib;

extern "C" {

TAD_API tad_status tad_newton_direction(tad_problem* P, const double* x_h, int projected, double eps, double w,
                                        double* d_h, double* f, double* g_h)
{
    if (!P || !x_h || !d_h) return fail(TAD_ERR_ARG, "NULL argument");
    if (!(w >= 0.0) || !std::isfinite(w)) return fail(TAD_ERR_ARG, "w_identity must be finite and non-negative");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    tad_status s = ensure_finalized(*P);
    if (s != TAD_OK) return s;
    TAD_CUDA_TRY(cudaMemcpyAsync(P->x, x_h, P->n_vars * 8, cudaMemcpyHostToDevice, P->stream));
    s = eval_full(*P, P->x, projected ? TAD_MODE_HESSIAN_PROJ : TAD_MODE_HESSIAN, eps, P->precision);
    if (s != TAD_OK) return s;
    if (w != 0.0) add_identity(*P, w, P->precision);   // H + w I (NewtonDirection.hh:32)
    k_neg<<<RED_BLOCKS, RED_THREADS, 0, P->stream>>>(P->n_vars, P->g, P->rhs);
    s = check_device_error(*P);
    if (s != TAD_OK) return s;
    int it = 0;
    tad_status ps = pcg_solve(*P, P->rhs, P->dx, 0.0, P->precision, P->settings.pcg_rel_tol, P->settings.pcg_max_iters, &it);
    if (ps != TAD_OK && ps != TAD_ERR_PCG_NOCONV) return ps;
    TAD_CUDA_TRY(cudaMemcpyAsync(d_h, P->dx, P->n_vars * 8, cudaMemcpyDeviceToHost, P->stream));
    if (g_h) TAD_CUDA_TRY(cudaMemcpyAsync(g_h, P->g, P->n_vars * 8, cudaMemcpyDeviceToHost, P->stream));
    TAD_CUDA_TRY(cudaMemcpyAsync(P->hs, P->ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, P->stream));
    TAD_CUDA_TRY(cudaStreamSynchronize(P->stream));
    if (f) *f = P->hs->f;
    P->pcg_iters_total = it;
    if (ps == TAD_ERR_PCG_NOCONV) set_error("Linear solve did not reach its tolerance.");
    return ps;
}

/* newton_decrement(d, g) = -d.g / 2 (include/TinyAD/Utils/NewtonDecrement.hh:20-26),
   as a fixed-order device reduction (k_dot_dg) on the problem's stream */
static tad_status newton_decrement_dev(Problem& P, const double* d_d, const double* g_d, double* out)
{
    cudaStream_t s = P.stream;
    k_dot_dg<<<RED_BLOCKS, RED_THREADS, 0, s>>>(P.n_vars, d_d, g_d, P.partials, P.counters + 4, P.ds);
    P.n_launches += 1;
    TAD_CUDA_TRY(cudaGetLastError());
    TAD_CUDA_TRY(cudaMemcpyAsync(P.hs, P.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, s));
    TAD_CUDA_TRY(cudaStreamSynchronize(s));
    *out = P.hs->decrement;
    return TAD_OK;
}

TAD_API tad_status tad_newton_decrement(tad_problem* P, const double* d_h, const double* g_h, double* out)
{
    if (!P || !d_h || !g_h || !out) return fail(TAD_ERR_ARG, "NULL argument");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    tad_status s = ensure_finalized(*P);
    if (s != TAD_OK) return s;
    const int64_t n = P->n_vars;
    // staged in the problem's own direction and right-hand-side buffers
    TAD_CUDA_TRY(cudaMemcpyAsync(P->dx, d_h, n * 8, cudaMemcpyHostToDevice, P->stream));
    TAD_CUDA_TRY(cudaMemcpyAsync(P->rhs, g_h, n * 8, cudaMemcpyHostToDevice, P->stream));
    return newton_decrement_dev(*P, P->dx, P->rhs, out);
}

TAD_API tad_status tad_newton_decrement_d(tad_problem* P, const double* d_d, const double* g_d, double* out)
{
    if (!P || !d_d || !g_d || !out) return fail(TAD_ERR_ARG, "NULL argument");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    tad_status s = ensure_finalized(*P);
    if (s != TAD_OK) return s;
    return newton_decrement_dev(*P, d_d, g_d, out);
}

TAD_API tad_status tad_line_search(tad_problem* P, const double* x_h, const double* d_h, double f, const double* g_h,
                                   double s_max, double* x_out_h, double* f_out)
{
    if (!P || !x_h || !d_h || !g_h || !x_out_h) return fail(TAD_ERR_ARG, "NULL argument");
    if (s_max <= 0.0) return fail(TAD_ERR_ARG, "Max step size not positive.");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    tad_status s = ensure_finalized(*P);
    if (s != TAD_OK) return s;
    const int64_t n = P->n_vars;
    TAD_CUDA_TRY(cudaMemcpyAsync(P->x, x_h, n * 8, cudaMemcpyHostToDevice, P->stream));
    TAD_CUDA_TRY(cudaMemcpyAsync(P->dx, d_h, n * 8, cudaMemcpyHostToDevice, P->stream));
    TAD_CUDA_TRY(cudaMemcpyAsync(P->g, g_h, n * 8, cudaMemcpyHostToDevice, P->stream));
    bool found = false;
    double fo = f;
    int trials = 0;
    s = line_search_device(*P, P->x, P->dx, f, s_max, &found, &fo, &trials);
    if (s != TAD_OK) return s;
    TAD_CUDA_TRY(cudaMemcpyAsync(x_out_h, P->x, n * 8, cudaMemcpyDeviceToHost, P->stream));
    TAD_CUDA_TRY(cudaStreamSynchronize(P->stream));
    if (f_out) *f_out = fo;
    P->ls_trials_total = trials;
    if (!found) { set_error("Line search couldn't find improvement."); return TAD_ERR_LS_FAIL; }
    return TAD_OK;
}

/* Time the main kernels once each at the current state (CUDA events on the
   problem's stream): [0] element Hessian kernels (all terms, current
   precision, projected), [1] Hessian + gradient assembly, [2] one PCG SpMV,
   [3] one PCG update, [4] line-search energy for one trial step. */
TAD_API tad_status tad_profile_kernels(tad_problem* P, const double* x_d, int reps, double* ms5)
{
    if (!P || !x_d || !ms5 || reps < 1) return fail(TAD_ERR_ARG, "bad argument");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    tad_status s = ensure_finalized(*P);
    if (s != TAD_OK) return s;
    Problem& Q = *P;
    cudaStream_t st = Q.stream;
    const int prec = Q.precision;
    // a valid state: Hessian at x, a search direction p = z = D^-1 g
    s = eval_full(Q, x_d, TAD_MODE_HESSIAN_PROJ, 1e-9, prec);
    if (s != TAD_OK) return s;
    k_neg<<<RED_BLOCKS, RED_THREADS, 0, st>>>(Q.n_vars, Q.g, Q.rhs);
    cudaEvent_t e0 = Q.ev[5], e1 = Q.ev[6];
    float ms = 0.f;
    // each kernel is timed as the solver runs it: reps launches captured in one
    // CUDA graph and replayed (the PCG's iterations run from captured graphs),
    // so the figure is the kernels' own time plus the graph's launch spacing;
    // launched from the host one by one they would add the launch latency
    auto timed = [&](auto&& launch) -> double {
        launch();   // warm
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        bool graph_ok = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (graph_ok)
        {
            for (int r = 0; r < reps; ++r) launch();
            graph_ok = cudaStreamEndCapture(st, &g) == cudaSuccess && cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
            if (graph_ok) graph_ok = cudaGraphLaunch(ge, st) == cudaSuccess;   // warm the graph
        }
        cudaGetLastError();
        cudaEventRecord(e0, st);
        if (graph_ok) cudaGraphLaunch(ge, st);
        else
            for (int r = 0; r < reps; ++r) launch();
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (ge) cudaGraphExecDestroy(ge);
        if (g) cudaGraphDestroy(g);
        return (double)ms / reps;
    };
    ms5[0] = timed([&] { eval_elements(Q, TAD_MODE_HESSIAN_PROJ, x_d, 1e-9, prec); });
    ms5[1] = timed([&] { launch_assemble_grad(Q, prec, prec == TAD_PREC_MIXED); launch_assemble_hess(Q, prec); });
    const int64_t nh = Q.n_handles, n = Q.n_vars;
#define TAD_PROF(D)                                                                                                  \
    if (prec == TAD_PREC_MIXED)                                                                                     \
    {                                                                                                               \
        k_pcg_init<D, float><<<RED_BLOCKS, RED_THREADS, 0, st>>>(nh, Q.rhs, Q.dx32, Q.r32, Q.z32, Q.p32, Q.Ap32,    \
                                                                 Q.dinv32, Q.diag, (const float*)Q.H, 0.0,         \
                                                                 Q.partials, Q.counters, Q.ds, 1e-30, 1 << 30);    \
        ms5[2] = timed([&] { launch_pcg_spmv<D, float>(st, sell_view(Q, (const float*)Q.H), nh, Q.bptr, Q.bcol, (const float*)Q.H, Q.z32, Q.p32,     \
                                                       Q.Ap32, Q.partials, Q.counters + 1, Q.ds); });                 \
        ms5[3] = timed([&] { k_pcg_update<D, float><<<RED_BLOCKS, RED_THREADS, 0, st>>>(nh, Q.dx32, Q.r32, Q.z32,  \
                               Q.p32, Q.Ap32, Q.dinv32, Q.partials, Q.counters + 2, Q.ds); });                       \
    }                                                                                                               \
    else                                                                                                            \
    {                                                                                                               \
        k_pcg_init<D, double><<<RED_BLOCKS, RED_THREADS, 0, st>>>(nh, Q.rhs, Q.dx, Q.r, Q.z, Q.p, Q.Ap, Q.dinv,     \
                                                                  Q.diag, (const double*)Q.H, 0.0,                  \
                                                                  Q.partials, Q.counters, Q.ds, 1e-30, 1 << 30);    \
        ms5[2] = timed([&] { launch_pcg_spmv<D, double>(st, sell_view(Q, (const double*)Q.H), nh, Q.bptr, Q.bcol, (const double*)Q.H, Q.z, Q.p, Q.Ap, \
                                                        Q.partials, Q.counters + 1, Q.ds); });                        \
        ms5[3] = timed([&] { k_pcg_update<D, double><<<RED_BLOCKS, RED_THREADS, 0, st>>>(nh, Q.dx, Q.r, Q.z,       \
                               Q.p, Q.Ap, Q.dinv, Q.partials, Q.counters + 2, Q.ds); });                             \
    }
    switch (Q.d)
    {
    case 1: TAD_PROF(1); break;
    case 2: TAD_PROF(2); break;
    default: TAD_PROF(3); break;
    }
#undef TAD_PROF
    // keep the PCG kernels from early-exiting: done was cleared by k_pcg_init with an unreachable tolerance
    const double one = 1.0;
    TAD_CUDA_TRY(cudaMemcpyAsync(Q.steps, &one, sizeof(double), cudaMemcpyHostToDevice, st));
    ms5[4] = timed([&] { eval_elements(Q, TAD_MODE_LINESEARCH, x_d, 0.0, Q.precision, Q.rhs, 1); });
    TAD_CUDA_TRY(cudaStreamSynchronize(st));
    TAD_CUDA_TRY(cudaGetLastError());
    return check_device_error(Q);
}

TAD_API tad_status tad_newton_solve_d(tad_problem* P, double* x_d, int n_iters, double eps, double stop_decrement,
                                      double* f_hist_h, int* iters_done)
{
    if (!P || !x_d) return fail(TAD_ERR_ARG, "NULL argument");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    return newton_solve(*P, x_d, n_iters, eps, stop_decrement, f_hist_h, iters_done);
}

TAD_API tad_status tad_newton_solve(tad_problem* P, double* x_h, int n_iters, double eps, double stop_decrement,
                                    double* f_hist_h, int* iters_done)
{
    if (!P || !x_h) return fail(TAD_ERR_ARG, "NULL argument");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    tad_status s = ensure_finalized(*P);
    if (s != TAD_OK) return s;
    // x is copied in and out by the solve, beside its compute where it can
    return newton_solve(*P, P->x, n_iters, eps, stop_decrement, f_hist_h, iters_done, x_h, x_h);
}

} // extern "C"
