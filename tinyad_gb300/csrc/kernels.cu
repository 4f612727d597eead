/*
 * Assembly and reduction kernels.  All of them are HBM-bound gathers; none
 * uses floating-point atomics, so every result is bitwise reproducible.
 *
 *   k_reduce_rows     f = sum of element energies (one row per line-search
 *                     trial), fixed partition over RED_BLOCKS blocks, then
 *                     the last block to finish sums the block partials in
 *                     block order.
 *   k_assemble_grad   g[v] = sum over v's element slots, in element order
 *                     (ScalarObjectiveTerm.hh:262-264 adds them in that order).
 *   k_assemble_hess   H block (u,w) = sum over its element pair blocks, in
 *                     element order (the order setFromTriplets sums
 *                     duplicates, ScalarFunctionImpl.hh:398).  Algorithmic
 *                     bytes per block: its contributions' d*d values + 4-byte
 *                     ids, plus d*d values written.
 *   k_bsr_to_csr      scalar CSR values (Eigen's CSC arrays for symmetric H)
 *                     from the BSR blocks, for the host-facing Hessian.
 */
#include "internal.hh"
#include "grid_reduce.cuh"
#include "../../include/tad/RowIO.cuh"
#include "../../include/tad/Scalar.cuh"

namespace tadlib {

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

/* fixed-order block sum; result valid in thread 0 */
__device__ __forceinline__ double block_sum(double v, double* sh)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    v = warp_sum(v);
    if (lane == 0) sh[w] = v;
    __syncthreads();
    v = 0.0;
    if (w == 0)
    {
        v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
        v = warp_sum(v);
    }
    __syncthreads();
    return v;
}

__global__ void __launch_bounds__(RED_THREADS) k_reduce_rows(const double* ef, int64_t n, int64_t stride,
                                                             double* partials, unsigned* counters, double* out)
{
    __shared__ double sh[32];
    __shared__ bool last;
    const int row = blockIdx.y;
    const double* a = ef + (int64_t)row * stride;
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t beg = (int64_t)blockIdx.x * chunk;
    const int64_t end = min(n, beg + chunk);
    double v = 0.0;
    for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) v += a[i];
    v = block_sum(v, sh);
    if (threadIdx.x == 0)
    {
        partials[(int64_t)row * gridDim.x + blockIdx.x] = v;
        __threadfence();
        const unsigned t = atomicAdd(&counters[row], 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += __ldcg(&partials[(int64_t)row * gridDim.x + i]);
    s = block_sum(s, sh);
    if (threadIdx.x == 0)
    {
        out[row] = s;
        counters[row] = 0u;
    }
}

void launch_reduce_f(Problem& P, int n_rows, double* out)
{
    const int64_t n = P.n_elem_total;
    int blocks = (int)std::min<int64_t>(RED_BLOCKS, std::max<int64_t>(1, (n + 4095) / 4096));
    dim3 grid(blocks, n_rows);
    k_reduce_rows<<<grid, RED_THREADS, 0, P.stream>>>(P.ef, n, n, P.partials, P.counters, out);
}

/* ---- gradient assembly -------------------------------------------------
   g[u] = sum of handle u's element gradient slots, in element order.  Acc =
   double (FP64 path) or tad::DoubleFloatValue (mixed: the double slot values
   are split bit-wise and summed on the FP32 pipe, ~48-bit, the precision of
   the mixed element gradients; FP64 adds bound this gather otherwise).
   Rows come from the length buckets (GatherBuckets): a thread loads its
   row's slot ids (coalesced across the warp, column-major), then the slot
   values, CH at a time, and sums them in order; rows longer than 64 slots
   use the CSR lists. */
template <int d, typename Acc, int W>
__device__ __forceinline__ void bucket_gather_grad(const int32_t* __restrict__ ids, int64_t stride, int64_t i,
                                                   const double* __restrict__ eg, Acc (&acc)[d])
{
    constexpr int CH = W < 4 ? W : 4;
#pragma unroll(W <= 8 ? W / CH : 1)
    for (int j0 = 0; j0 < W; j0 += CH)
    {
        int32_t c[CH];
#pragma unroll
        for (int jj = 0; jj < CH; ++jj) c[jj] = ids[(int64_t)(j0 + jj) * stride + i];
        if (c[0] < 0) break;   // padding follows a row's slots
        double v[CH][d];
#pragma unroll
        for (int jj = 0; jj < CH; ++jj)
            if (c[jj] >= 0)
            {
#pragma unroll
                for (int p = 0; p < d; ++p) v[jj][p] = eg[(int64_t)c[jj] * d + p];
            }
#pragma unroll
        for (int jj = 0; jj < CH; ++jj)
        {
            if (c[jj] < 0) break;
#pragma unroll
            for (int p = 0; p < d; ++p) acc[p] = acc[p] + Acc(v[jj][p]);
        }
    }
}

template <int d, typename Acc>
__device__ __forceinline__ void csr_gather_grad(int64_t u, const int32_t* __restrict__ gptr, const int32_t* __restrict__ gidx,
                                                const double* __restrict__ eg, Acc (&acc)[d])
{
    for (int32_t q = gptr[u]; q < gptr[u + 1]; ++q)
    {
        const int64_t sl = gidx[q];
#pragma unroll
        for (int p = 0; p < d; ++p) acc[p] = acc[p] + Acc(eg[sl * d + p]);
    }
}

/* bucket b of padded row t, its index i within the bucket, the bucket's row
   count (the id stride) and id base, selected with unrolled compares so the
   kernel parameter stays in constant memory */
__device__ __forceinline__ void bucket_of_row(const GatherBuckets& B, int64_t t, int& b, int64_t& i, int64_t& stride,
                                              const int32_t*& ids)
{
    b = 0;
    int64_t lo = B.row_begin[0], hi = B.row_begin[1], ib = B.id_begin[0];
#pragma unroll
    for (int q = 1; q < GATHER_BUCKETS; ++q)
        if (t >= B.row_begin[q])
        {
            b = q;
            lo = B.row_begin[q];
            hi = B.row_begin[q + 1];
            ib = B.id_begin[q];
        }
    i = t - lo;
    stride = hi - lo;
    ids = B.ids + ib;
}

/* row t of the bucket list (t < padded rows) or long row t - padded; returns
   the output row (-1 for padding) and the sum */
template <int d, typename Acc>
__device__ __forceinline__ int64_t gather_grad_row(int64_t t, const GatherBuckets& B, const int32_t* __restrict__ gptr,
                                                   const int32_t* __restrict__ gidx, const double* __restrict__ eg,
                                                   double (&out)[d])
{
    Acc acc[d];
#pragma unroll
    for (int p = 0; p < d; ++p) acc[p] = Acc(0.0);
    const int64_t padded = B.row_begin[GATHER_BUCKETS];
    int64_t r;
    if (t < padded)
    {
        int b;
        int64_t i, stride;
        const int32_t* ids;
        bucket_of_row(B, t, b, i, stride, ids);
        switch (b)
        {
        case 0: bucket_gather_grad<d, Acc, 1>(ids, stride, i, eg, acc); break;
        case 1: bucket_gather_grad<d, Acc, 2>(ids, stride, i, eg, acc); break;
        case 2: bucket_gather_grad<d, Acc, 4>(ids, stride, i, eg, acc); break;
        case 3: bucket_gather_grad<d, Acc, 8>(ids, stride, i, eg, acc); break;
        case 4: bucket_gather_grad<d, Acc, 16>(ids, stride, i, eg, acc); break;
        case 5: bucket_gather_grad<d, Acc, 32>(ids, stride, i, eg, acc); break;
        default: bucket_gather_grad<d, Acc, 64>(ids, stride, i, eg, acc); break;
        }
        r = B.rows[t];
    }
    else
    {
        r = B.long_rows[t - padded];
        csr_gather_grad<d, Acc>(r, gptr, gidx, eg, acc);
    }
#pragma unroll
    for (int p = 0; p < d; ++p) out[p] = (double)acc[p];
    return r;
}

template <int d, typename Acc>
__global__ void __launch_bounds__(256) k_assemble_grad(GatherBuckets B, const int32_t* __restrict__ gptr,
                                                       const int32_t* __restrict__ gidx, const double* __restrict__ eg,
                                                       double* __restrict__ g)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= B.row_begin[GATHER_BUCKETS] + B.n_long) return;
    double gv[d];
    const int64_t r = gather_grad_row<d, Acc>(t, B, gptr, gidx, eg, gv);
    if (r < 0) return;
#pragma unroll
    for (int p = 0; p < d; ++p) g[r * d + p] = gv[p];
}

/* The Newton variant: also rhs = -g and g.g (the PCG right-hand side and
   |g|^2), one thread per row, block partials summed in block order by the
   last block (the partials buffer holds one per block) */
template <int d, typename Acc>
__global__ void __launch_bounds__(RED_THREADS) k_assemble_grad_newton(GatherBuckets B, const int32_t* __restrict__ gptr,
                                                                    const int32_t* __restrict__ gidx,
                                                                    const double* __restrict__ eg, double* __restrict__ g,
                                                                    double* __restrict__ rhs, double* partials,
                                                                    unsigned* counter, DevScalars* ds)
{
    double part[1] = {0.0};
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < B.row_begin[GATHER_BUCKETS] + B.n_long)
    {
        double gv[d];
        const int64_t r = gather_grad_row<d, Acc>(t, B, gptr, gidx, eg, gv);
        if (r >= 0)
        {
#pragma unroll
            for (int p = 0; p < d; ++p)
            {
                g[r * d + p] = gv[p];
                rhs[r * d + p] = -gv[p];
                part[0] += gv[p] * gv[p];
            }
        }
    }
    double tot[1];
    if (!grid_sum<1>(part, partials, counter, tot)) return;
    if (threadIdx.x == 0) ds->gg = tot[0];
}

template <typename Acc>
static void assemble_grad_as(Problem& P)
{
    const int64_t rows = P.grad_buckets.row_begin[GATHER_BUCKETS] + P.grad_buckets.n_long;
    if (rows == 0) return;
    const unsigned grid = (unsigned)((rows + 255) / 256);
    switch (P.d)
    {
    case 1: k_assemble_grad<1, Acc><<<grid, 256, 0, P.stream>>>(P.grad_buckets, P.gptr, P.gidx, P.eg, P.g); break;
    case 2: k_assemble_grad<2, Acc><<<grid, 256, 0, P.stream>>>(P.grad_buckets, P.gptr, P.gidx, P.eg, P.g); break;
    default: k_assemble_grad<3, Acc><<<grid, 256, 0, P.stream>>>(P.grad_buckets, P.gptr, P.gidx, P.eg, P.g); break;
    }
}

void launch_assemble_grad(Problem& P, int precision)
{
    if (precision == TAD_PREC_MIXED) assemble_grad_as<tad::DoubleFloatValue>(P);
    else assemble_grad_as<double>(P);
}

template <typename Acc>
static void assemble_grad_newton_as(Problem& P)
{
    const int64_t rows = P.grad_buckets.row_begin[GATHER_BUCKETS] + P.grad_buckets.n_long;
    const unsigned grid = (unsigned)std::max<int64_t>(1, (rows + RED_THREADS - 1) / RED_THREADS);   // <= partials_cap
    switch (P.d)
    {
    case 1: k_assemble_grad_newton<1, Acc><<<grid, RED_THREADS, 0, P.stream>>>(P.grad_buckets, P.gptr, P.gidx, P.eg, P.g, P.rhs,
                                                                               P.partials, P.counters + 5, P.ds); break;
    case 2: k_assemble_grad_newton<2, Acc><<<grid, RED_THREADS, 0, P.stream>>>(P.grad_buckets, P.gptr, P.gidx, P.eg, P.g, P.rhs,
                                                                               P.partials, P.counters + 5, P.ds); break;
    default: k_assemble_grad_newton<3, Acc><<<grid, RED_THREADS, 0, P.stream>>>(P.grad_buckets, P.gptr, P.gidx, P.eg, P.g, P.rhs,
                                                                                P.partials, P.counters + 5, P.ds); break;
    }
}

void launch_assemble_grad_newton(Problem& P, int precision)
{
    if (precision == TAD_PREC_MIXED) assemble_grad_newton_as<tad::DoubleFloatValue>(P);
    else assemble_grad_newton_as<double>(P);
}

/* ---- Hessian assembly ---------------------------------------------------
   H block (u, w) = sum of its element pair blocks in element order (bit 31 of
   an id: the element block is stored transposed).  Same bucket scheme. */
template <int d, typename T>
__device__ __forceinline__ void add_block(T (&acc)[d * d], const T (&v)[d * d], bool transposed)
{
    if (transposed)
    {
#pragma unroll
        for (int p = 0; p < d; ++p)
#pragma unroll
            for (int r = 0; r < d; ++r) acc[p * d + r] += v[r * d + p];
    }
    else
    {
#pragma unroll
        for (int i = 0; i < d * d; ++i) acc[i] += v[i];
    }
}

template <int d, typename T, int W>
__device__ __forceinline__ void bucket_gather_hess(const int32_t* __restrict__ ids, int64_t stride, int64_t i,
                                                   const T* __restrict__ eH, T (&acc)[d * d])
{
    constexpr int CH = W < 4 ? W : 4;
#pragma unroll(W <= 8 ? W / CH : 1)
    for (int j0 = 0; j0 < W; j0 += CH)
    {
        int32_t c[CH];
#pragma unroll
        for (int jj = 0; jj < CH; ++jj) c[jj] = ids[(int64_t)(j0 + jj) * stride + i];
        if (c[0] == -1) break;   // padding follows a row's contributions
        T v[CH][d * d];
#pragma unroll
        for (int jj = 0; jj < CH; ++jj)
            if (c[jj] != -1) tad::load_row<T, d * d>(eH, (int64_t)(c[jj] & 0x7fffffff), v[jj]);   // 16-byte load per 2x2 FP32 block
#pragma unroll
        for (int jj = 0; jj < CH; ++jj)
        {
            if (c[jj] == -1) break;
            add_block<d, T>(acc, v[jj], c[jj] < 0);
        }
    }
}

template <int d, typename T>
__global__ void __launch_bounds__(256) k_assemble_hess(GatherBuckets B, const int32_t* __restrict__ cptr,
                                                       const int32_t* __restrict__ cidx, const T* __restrict__ eH,
                                                       T* __restrict__ H)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t padded = B.row_begin[GATHER_BUCKETS];
    if (t >= padded + B.n_long) return;
    T acc[d * d];
#pragma unroll
    for (int i = 0; i < d * d; ++i) acc[i] = T(0);
    int64_t r;
    if (t < padded)
    {
        int b;
        int64_t i, stride;
        const int32_t* ids;
        bucket_of_row(B, t, b, i, stride, ids);
        switch (b)
        {
        case 0: bucket_gather_hess<d, T, 1>(ids, stride, i, eH, acc); break;
        case 1: bucket_gather_hess<d, T, 2>(ids, stride, i, eH, acc); break;
        case 2: bucket_gather_hess<d, T, 4>(ids, stride, i, eH, acc); break;
        case 3: bucket_gather_hess<d, T, 8>(ids, stride, i, eH, acc); break;
        case 4: bucket_gather_hess<d, T, 16>(ids, stride, i, eH, acc); break;
        case 5: bucket_gather_hess<d, T, 32>(ids, stride, i, eH, acc); break;
        default: bucket_gather_hess<d, T, 64>(ids, stride, i, eH, acc); break;
        }
        r = B.rows[t];
        if (r < 0) return;
    }
    else
    {
        r = B.long_rows[t - padded];
        for (int32_t q = cptr[r]; q < cptr[r + 1]; ++q)
        {
            const int32_t c = cidx[q];
            T v[d * d];
            tad::load_row<T, d * d>(eH, (int64_t)(c & 0x7fffffff), v);
            add_block<d, T>(acc, v, c < 0);
        }
    }
    tad::store_row<T, d * d>(H, r, acc);
}

void launch_assemble_hess(Problem& P, int precision)
{
    const int64_t rows = P.hess_buckets.row_begin[GATHER_BUCKETS] + P.hess_buckets.n_long;
    if (P.nb == 0 || rows == 0) return;
    const unsigned grid = (unsigned)((rows + 255) / 256);
#define TAD_ASM(D)                                                                                                   \
    if (precision == TAD_PREC_MIXED)                                                                                 \
        k_assemble_hess<D, float><<<grid, 256, 0, P.stream>>>(P.hess_buckets, P.cptr, P.cidx, (const float*)P.eH,    \
                                                              (float*)P.H);                                          \
    else                                                                                                             \
        k_assemble_hess<D, double><<<grid, 256, 0, P.stream>>>(P.hess_buckets, P.cptr, P.cidx, (const double*)P.eH,  \
                                                               (double*)P.H);
    switch (P.d)
    {
    case 1: TAD_ASM(1); break;
    case 2: TAD_ASM(2); break;
    default: TAD_ASM(3); break;
    }
#undef TAD_ASM
}

template <int d, typename T>
__global__ void k_bsr_to_csr(int64_t nh, const int32_t* __restrict__ bptr, const T* __restrict__ H, double* __restrict__ out)
{
    const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (u >= nh) return;
    const int32_t b0 = bptr[u];
    const int32_t nbr = bptr[u + 1] - b0;
    const int64_t base = (int64_t)d * d * b0;
    for (int32_t j = 0; j < nbr; ++j)
#pragma unroll
        for (int p = 0; p < d; ++p)
#pragma unroll
            for (int q = 0; q < d; ++q)
                out[base + (int64_t)p * d * nbr + j * d + q] = (double)H[(int64_t)(b0 + j) * d * d + p * d + q];
}

void launch_bsr_to_csr(Problem& P, double* out, int precision)
{
    const unsigned grid = (unsigned)((P.n_handles + 255) / 256);
#define TAD_B2C(D)                                                                                      \
    if (precision == TAD_PREC_MIXED)                                                                    \
        k_bsr_to_csr<D, float><<<grid, 256, 0, P.stream>>>(P.n_handles, P.bptr, (const float*)P.H, out); \
    else                                                                                                \
        k_bsr_to_csr<D, double><<<grid, 256, 0, P.stream>>>(P.n_handles, P.bptr, (const double*)P.H, out);
    switch (P.d)
    {
    case 1: TAD_B2C(1); break;
    case 2: TAD_B2C(2); break;
    default: TAD_B2C(3); break;
    }
#undef TAD_B2C
}

__global__ void k_zero(double* p, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = 0.0;
}

void launch_zero(double* p, int64_t n, cudaStream_t s)
{
    k_zero<<<RED_BLOCKS, RED_THREADS, 0, s>>>(p, n);
}

} // namespace tadlib
