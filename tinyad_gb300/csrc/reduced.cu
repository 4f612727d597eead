/*
 * Newton direction in a linear subspace (newton_direction_reduced_basis,
 * include/TinyAD/Utils/NewtonDirection.hh:76-123):
 *
 *   d = B (B^T H B + w I)^-1 (-B^T g),   B the n x m basis of the subspace,
 *
 * typically the free coordinates of a problem with fixed vertices, or a
 * constraint null space.  The reference forms B^T H B with sparse products
 * and factorises it; here the reduced system is solved matrix-free: each
 * CG iteration applies B (CSR SpMV), H (the assembled BSR Hessian, in its
 * stored precision, FP64 accumulation) and B^T (CSR of the transpose, built
 * once per call), with the exact diagonal of B^T H B as Jacobi
 * preconditioner.  The CG scalars live on the device (last-block grid
 * sums, fixed order, bitwise reproducible); every kernel returns at once
 * when the stop flag is set, and the host checks the flag once per chunk of
 * iterations.
 */
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.hh"
#include "grid_reduce.cuh"

namespace tadlib {

static tad_status fail(tad_status s, const char* m) { set_error(m); return s; }

struct RedScalars
{
    double rz, alpha, beta, bb, rr, tol2;
    int32_t done, iters, max_iters, breakdown;
};

/* y = A x for a CSR matrix (FP64) */
__global__ void k_red_csr(int64_t rows, const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                          const double* __restrict__ val, const double* __restrict__ x, double* __restrict__ y,
                          const RedScalars* rs)
{
    if (rs && *(volatile const int32_t*)&rs->done) return;
    GRID_STRIDE(i, rows)
    {
        double acc = 0.0;
        for (int32_t q = ptr[i]; q < ptr[i + 1]; ++q) acc += val[q] * x[idx[q]];
        y[i] = acc;
    }
}

/* v = H u, H the BSR Hessian (d x d blocks of T), FP64 accumulation */
template <int d, typename T>
__global__ void k_red_bsr(int64_t nh, const int32_t* __restrict__ bptr, const int32_t* __restrict__ bcol,
                          const T* __restrict__ H, const double* __restrict__ u, double* __restrict__ v, const RedScalars* rs)
{
    if (*(volatile const int32_t*)&rs->done) return;
    GRID_STRIDE(r, nh)
    {
        double y[d];
#pragma unroll
        for (int i = 0; i < d; ++i) y[i] = 0.0;
        for (int32_t b = bptr[r]; b < bptr[r + 1]; ++b)
        {
            const int64_t c = bcol[b];
#pragma unroll
            for (int i = 0; i < d; ++i)
#pragma unroll
                for (int j = 0; j < d; ++j) y[i] += (double)H[(int64_t)b * d * d + i * d + j] * u[c * d + j];
        }
#pragma unroll
        for (int i = 0; i < d; ++i) v[r * d + i] = y[i];
    }
}

/* the exact diagonal of B^T H B + w I, inverted (Jacobi preconditioner):
   column j of B holds entries (i, B_ij); diag_j = sum_{i,k} B_ij B_kj H(i, k) */
template <int d, typename T>
__global__ void k_red_diag(int64_t m, const int32_t* __restrict__ tptr, const int32_t* __restrict__ tidx,
                           const double* __restrict__ tval, const int32_t* __restrict__ bptr,
                           const int32_t* __restrict__ bcol, const T* __restrict__ H, double w, double* __restrict__ dinv)
{
    GRID_STRIDE(j, m)
    {
        double acc = w;
        for (int32_t a = tptr[j]; a < tptr[j + 1]; ++a)
        {
            const int32_t i = tidx[a];
            const int32_t br = i / d, pi = i % d;
            for (int32_t c = tptr[j]; c < tptr[j + 1]; ++c)
            {
                const int32_t k = tidx[c];
                const int32_t bc = k / d, pk = k % d;
                // block (br, bc): column ids of a block row are sorted
                int32_t lo = bptr[br], hi = bptr[br + 1];
                while (lo < hi)
                {
                    const int32_t mid = (lo + hi) >> 1;
                    if (bcol[mid] < bc) lo = mid + 1;
                    else hi = mid;
                }
                if (lo < bptr[br + 1] && bcol[lo] == bc)
                    acc += tval[a] * tval[c] * (double)H[(int64_t)lo * d * d + pi * d + pk];
            }
        }
        dinv[j] = (acc > 0.0 && isfinite(acc)) ? 1.0 / acc : 1.0;
    }
}

/* r = -B^T g, z = M^-1 r, p = z, x = 0; rz = r.z, bb = r.r */
__global__ void __launch_bounds__(RED_THREADS) k_red_init(int64_t m, const int32_t* __restrict__ tptr,
                                                          const int32_t* __restrict__ tidx, const double* __restrict__ tval,
                                                          const double* __restrict__ g, const double* __restrict__ dinv,
                                                          double* x, double* r, double* z, double* p, double* partials,
                                                          unsigned* counter, RedScalars* rs, double rel_tol, int max_iters)
{
    double part[2] = {0.0, 0.0};
    GRID_STRIDE(j, m)
    {
        double acc = 0.0;
        for (int32_t a = tptr[j]; a < tptr[j + 1]; ++a) acc -= tval[a] * g[tidx[a]];
        const double zj = acc * dinv[j];
        x[j] = 0.0;
        r[j] = acc;
        z[j] = zj;
        p[j] = zj;
        part[0] += acc * zj;
        part[1] += acc * acc;
    }
    double tot[2];
    if (!grid_sum<2>(part, partials, counter, tot)) return;
    if (threadIdx.x == 0)
    {
        rs->rz = tot[0];
        rs->bb = tot[1];
        rs->rr = tot[1];
        rs->tol2 = rel_tol * rel_tol * tot[1];
        rs->iters = 0;
        rs->breakdown = 0;
        rs->max_iters = max_iters;
        rs->done = (tot[1] == 0.0) ? 1 : 0;
    }
}

/* q = B^T v + w p; p.q; the last block sets alpha (or the breakdown flag) */
__global__ void __launch_bounds__(RED_THREADS) k_red_q(int64_t m, const int32_t* __restrict__ tptr,
                                                       const int32_t* __restrict__ tidx, const double* __restrict__ tval,
                                                       const double* __restrict__ v, const double* __restrict__ p, double w,
                                                       double* __restrict__ q, double* partials, unsigned* counter,
                                                       RedScalars* rs)
{
    if (*(volatile int32_t*)&rs->done) return;
    double part[1] = {0.0};
    GRID_STRIDE(j, m)
    {
        double acc = w * p[j];
        for (int32_t a = tptr[j]; a < tptr[j + 1]; ++a) acc += tval[a] * v[tidx[a]];
        q[j] = acc;
        part[0] += p[j] * acc;
    }
    double tot[1];
    if (!grid_sum<1>(part, partials, counter, tot)) return;
    if (threadIdx.x == 0)
    {
        if (!(tot[0] > 0.0)) { rs->breakdown = 1; rs->done = 1; rs->alpha = 0.0; }
        else rs->alpha = rs->rz / tot[0];
    }
}

/* x += alpha p, r -= alpha q, z = M^-1 r; r.z, r.r; the last block sets beta,
   counts the iteration and raises the stop flag */
__global__ void __launch_bounds__(RED_THREADS) k_red_update(int64_t m, double* x, double* r, double* z,
                                                            const double* __restrict__ p, const double* __restrict__ q,
                                                            const double* __restrict__ dinv, double* partials,
                                                            unsigned* counter, RedScalars* rs)
{
    if (*(volatile int32_t*)&rs->done) return;
    const double alpha = rs->alpha;
    double part[2] = {0.0, 0.0};
    GRID_STRIDE(j, m)
    {
        x[j] += alpha * p[j];
        const double rj = r[j] - alpha * q[j];
        r[j] = rj;
        const double zj = rj * dinv[j];
        z[j] = zj;
        part[0] += rj * zj;
        part[1] += rj * rj;
    }
    double tot[2];
    if (!grid_sum<2>(part, partials, counter, tot)) return;
    if (threadIdx.x == 0)
    {
        rs->beta = tot[0] / rs->rz;
        rs->rz = tot[0];
        rs->rr = tot[1];
        rs->iters += 1;
        if (tot[1] <= rs->tol2 || rs->iters >= rs->max_iters) rs->done = 1;
    }
}

/* p = z + beta p */
__global__ void k_red_p(int64_t m, const double* __restrict__ z, double* __restrict__ p, const RedScalars* rs)
{
    if (*(volatile const int32_t*)&rs->done) return;
    const double beta = rs->beta;
    GRID_STRIDE(j, m) p[j] = z[j] + beta * p[j];
}

struct DevBuf
{
    std::vector<void*> ptrs;
    template <typename T>
    cudaError_t alloc(T** p, size_t n)
    {
        const cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
        if (e == cudaSuccess) ptrs.push_back((void*)*p);
        return e;
    }
    ~DevBuf()
    {
        for (void* p : ptrs) cudaFree(p);
    }
};

template <int d, typename T>
static tad_status reduced_solve(Problem& P, int64_t m, const int32_t* b_outer, const int32_t* b_inner,
                                const double* b_values, double w, double* d_out, int* iters_out, bool* breakdown)
{
    const int64_t n = P.n_vars;
    cudaStream_t s = P.stream;
    const int64_t nnz = b_outer[n];
    // B^T as CSR (counting sort by column), entries of a column in row order
    std::vector<int32_t> tptr(m + 1, 0), tidx(nnz);
    std::vector<double> tval(nnz);
    for (int64_t q = 0; q < nnz; ++q) ++tptr[b_inner[q] + 1];
    for (int64_t j = 0; j < m; ++j) tptr[j + 1] += tptr[j];
    {
        std::vector<int32_t> fill(tptr.begin(), tptr.end() - 1);
        for (int64_t i = 0; i < n; ++i)
            for (int32_t q = b_outer[i]; q < b_outer[i + 1]; ++q)
            {
                const int32_t at = fill[b_inner[q]]++;
                tidx[at] = (int32_t)i;
                tval[at] = b_values[q];
            }
    }
    DevBuf buf;
    int32_t *bo = nullptr, *bi = nullptr, *to = nullptr, *ti = nullptr;
    double *bv = nullptr, *tv = nullptr, *xr = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
    double *u = nullptr, *v = nullptr, *dinv = nullptr, *dd = nullptr;
    RedScalars* rs = nullptr;
    TAD_CUDA_TRY(buf.alloc(&bo, n + 1));
    TAD_CUDA_TRY(buf.alloc(&bi, nnz));
    TAD_CUDA_TRY(buf.alloc(&bv, nnz));
    TAD_CUDA_TRY(buf.alloc(&to, m + 1));
    TAD_CUDA_TRY(buf.alloc(&ti, nnz));
    TAD_CUDA_TRY(buf.alloc(&tv, nnz));
    for (double** a : {&xr, &r, &z, &p, &q, &dinv}) TAD_CUDA_TRY(buf.alloc(a, m));
    for (double** a : {&u, &v, &dd}) TAD_CUDA_TRY(buf.alloc(a, n));
    TAD_CUDA_TRY(buf.alloc(&rs, 1));
    TAD_CUDA_TRY(cudaMemcpyAsync(bo, b_outer, (n + 1) * 4, cudaMemcpyHostToDevice, s));
    TAD_CUDA_TRY(cudaMemcpyAsync(bi, b_inner, nnz * 4, cudaMemcpyHostToDevice, s));
    TAD_CUDA_TRY(cudaMemcpyAsync(bv, b_values, nnz * 8, cudaMemcpyHostToDevice, s));
    TAD_CUDA_TRY(cudaMemcpyAsync(to, tptr.data(), (m + 1) * 4, cudaMemcpyHostToDevice, s));
    TAD_CUDA_TRY(cudaMemcpyAsync(ti, tidx.data(), nnz * 4, cudaMemcpyHostToDevice, s));
    TAD_CUDA_TRY(cudaMemcpyAsync(tv, tval.data(), nnz * 8, cudaMemcpyHostToDevice, s));
    const T* H = (const T*)P.H;
    k_red_diag<d, T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(m, to, ti, tv, P.bptr, P.bcol, H, w, dinv);
    k_red_init<<<RED_BLOCKS, RED_THREADS, 0, s>>>(m, to, ti, tv, P.g, dinv, xr, r, z, p, P.partials, P.counters + 6, rs,
                                                  P.settings.pcg_rel_tol, std::max(1, P.settings.pcg_max_iters));
    P.n_launches += 2;
    TAD_CUDA_TRY(cudaGetLastError());
    RedScalars h{};
    constexpr int CHUNK = 8;
    for (;;)
    {
        for (int it = 0; it < CHUNK; ++it)
        {
            k_red_csr<<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, bo, bi, bv, p, u, rs);
            k_red_bsr<d, T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(P.n_handles, P.bptr, P.bcol, H, u, v, rs);
            k_red_q<<<RED_BLOCKS, RED_THREADS, 0, s>>>(m, to, ti, tv, v, p, w, q, P.partials, P.counters + 7, rs);
            k_red_update<<<RED_BLOCKS, RED_THREADS, 0, s>>>(m, xr, r, z, p, q, dinv, P.partials, P.counters + 8, rs);
            k_red_p<<<RED_BLOCKS, RED_THREADS, 0, s>>>(m, z, p, rs);
        }
        P.n_launches += 5 * CHUNK;
        TAD_CUDA_TRY(cudaGetLastError());
        TAD_CUDA_TRY(cudaMemcpyAsync(&h, rs, sizeof(RedScalars), cudaMemcpyDeviceToHost, s));
        TAD_CUDA_TRY(cudaStreamSynchronize(s));
        if (h.done) break;
    }
    // d = B x_r
    k_red_csr<<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, bo, bi, bv, xr, dd, nullptr);
    P.n_launches += 1;
    TAD_CUDA_TRY(cudaMemcpyAsync(d_out, dd, n * 8, cudaMemcpyDeviceToHost, s));
    TAD_CUDA_TRY(cudaStreamSynchronize(s));
    *iters_out = h.iters;
    *breakdown = h.breakdown != 0;
    if (h.breakdown) return TAD_ERR_PCG_NOCONV;
    return (h.rr <= h.tol2) ? TAD_OK : TAD_ERR_PCG_NOCONV;
}

} // namespace tadlib

using namespace tadlib;

extern "C" TAD_API tad_status tad_newton_direction_reduced_basis(tad_problem* P, const double* x_h, int64_t m,
                                                                 const int32_t* b_outer, const int32_t* b_inner,
                                                                 const double* b_values, double eps, double w,
                                                                 double* d_h, double* f, double* g_h)
{
    if (!P || !x_h || !b_outer || !d_h || m < 0) return fail(TAD_ERR_ARG, "NULL argument");
    if (w < 0.0 || !std::isfinite(w)) return fail(TAD_ERR_ARG, "w_identity must be finite and non-negative");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    tad_status s = ensure_finalized(*P);
    if (s != TAD_OK) return s;
    const int64_t n = P->n_vars;
    if (b_outer[0] != 0) return fail(TAD_ERR_ARG, "basis: outer[0] must be 0");
    for (int64_t i = 0; i < n; ++i)
        if (b_outer[i + 1] < b_outer[i]) return fail(TAD_ERR_ARG, "basis: outer indices must not decrease");
    const int64_t nnz = b_outer[n];
    if (nnz > 0 && (!b_inner || !b_values)) return fail(TAD_ERR_ARG, "NULL argument");
    for (int64_t q = 0; q < nnz; ++q)
        if (b_inner[q] < 0 || b_inner[q] >= m) return fail(TAD_ERR_ARG, "basis: column index out of range");
    TAD_CUDA_TRY(cudaMemcpyAsync(P->x, x_h, n * 8, cudaMemcpyHostToDevice, P->stream));
    s = eval_full(*P, P->x, TAD_MODE_HESSIAN_PROJ, eps, P->precision);
    if (s != TAD_OK) return s;
    s = check_device_error(*P);
    if (s != TAD_OK) return s;
    int iters = 0;
    bool breakdown = false;
    tad_status ps = TAD_OK;
    const bool fp32 = P->precision == TAD_PREC_MIXED;
    switch (P->d)
    {
    case 1: ps = fp32 ? reduced_solve<1, float>(*P, m, b_outer, b_inner, b_values, w, d_h, &iters, &breakdown)
                      : reduced_solve<1, double>(*P, m, b_outer, b_inner, b_values, w, d_h, &iters, &breakdown); break;
    case 2: ps = fp32 ? reduced_solve<2, float>(*P, m, b_outer, b_inner, b_values, w, d_h, &iters, &breakdown)
                      : reduced_solve<2, double>(*P, m, b_outer, b_inner, b_values, w, d_h, &iters, &breakdown); break;
    default: ps = fp32 ? reduced_solve<3, float>(*P, m, b_outer, b_inner, b_values, w, d_h, &iters, &breakdown)
                       : reduced_solve<3, double>(*P, m, b_outer, b_inner, b_values, w, d_h, &iters, &breakdown); break;
    }
    if (ps != TAD_OK && ps != TAD_ERR_PCG_NOCONV) return ps;
    if (g_h) TAD_CUDA_TRY(cudaMemcpyAsync(g_h, P->g, n * 8, cudaMemcpyDeviceToHost, P->stream));
    TAD_CUDA_TRY(cudaMemcpyAsync(P->hs, P->ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, P->stream));
    TAD_CUDA_TRY(cudaStreamSynchronize(P->stream));
    if (f) *f = P->hs->f;
    P->pcg_iters_total = iters;
    if (ps == TAD_ERR_PCG_NOCONV)
        set_error(breakdown ? "Linear solve failed (non-positive curvature in the reduced system)."
                            : "Linear solve did not reach its tolerance.");
    return ps;
}
