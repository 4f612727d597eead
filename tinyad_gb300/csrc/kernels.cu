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
                                                             double* partials, unsigned* counters, double* out,
                                                             const int32_t* guard)
{
    if (guard && *guard == 0) return;   // every block returns before touching the counters
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
    k_reduce_rows<<<grid, RED_THREADS, 0, P.stream>>>(P.ef, n, n, P.partials, P.counters, out, P.launch_guard);
}

/* g[u] = sum of handle u's element gradient slots, in element order.  Acc =
   double (FP64 path) or tad::DoubleFloatValue (mixed: the double slot values
   are split bit-wise and summed on the FP32 pipe, ~48-bit, the precision of
   the mixed element gradients; FP64 adds bound this gather otherwise).
   Slots are gathered in batches of GATHER (ids, then values, loaded
   together) and summed in order. */
template <int d, typename Acc, bool Pairs>
__device__ __forceinline__ void gather_gradient(int64_t u, const int32_t* __restrict__ gptr, const int32_t* __restrict__ gidx,
                                                const double* __restrict__ eg, double (&out)[d])
{
    // Pairs: the slots hold double-float pairs (mixed second-order modes)
    const float2* __restrict__ eg2 = reinterpret_cast<const float2*>(eg);
    Acc acc[d];
#pragma unroll
    for (int p = 0; p < d; ++p) acc[p] = Acc(0.0);
    constexpr int GATHER = 4;
    const int32_t q0 = gptr[u], q1 = gptr[u + 1];
    for (int32_t q = q0; q < q1; q += GATHER)
    {
        int64_t sl[GATHER];
#pragma unroll
        for (int j = 0; j < GATHER; ++j) sl[j] = (q + j < q1) ? gidx[q + j] : 0;
        if constexpr (Pairs)
        {
            float2 v[GATHER][d];
#pragma unroll
            for (int j = 0; j < GATHER; ++j)
                if (q + j < q1)
                {
#pragma unroll
                    for (int p = 0; p < d; ++p) v[j][p] = eg2[sl[j] * d + p];
                }
#pragma unroll
            for (int j = 0; j < GATHER; ++j)
            {
                if (q + j >= q1) break;
#pragma unroll
                for (int p = 0; p < d; ++p) acc[p] = acc[p] + tad::DoubleFloatValue(v[j][p].x, v[j][p].y);
            }
        }
        else
        {
            double v[GATHER][d];
#pragma unroll
            for (int j = 0; j < GATHER; ++j)
                if (q + j < q1)
                {
#pragma unroll
                    for (int p = 0; p < d; ++p) v[j][p] = eg[sl[j] * d + p];
                }
#pragma unroll
            for (int j = 0; j < GATHER; ++j)
            {
                if (q + j >= q1) break;
#pragma unroll
                for (int p = 0; p < d; ++p) acc[p] = acc[p] + Acc(v[j][p]);
            }
        }
    }
#pragma unroll
    for (int p = 0; p < d; ++p) out[p] = (double)acc[p];
}

template <int d, typename Acc, bool Pairs>
__global__ void k_assemble_grad(int64_t nh, const int32_t* __restrict__ gptr, const int32_t* __restrict__ gidx,
                                const double* __restrict__ eg, double* __restrict__ g)
{
    const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (u >= nh) return;
    double gv[d];
    gather_gradient<d, Acc, Pairs>(u, gptr, gidx, eg, gv);
#pragma unroll
    for (int p = 0; p < d; ++p) g[u * d + p] = gv[p];
}

/* The Newton variant: also rhs = -g and g.g (the PCG right-hand side and
   |g|^2), grid-stride over a capped grid for the fixed-order grid sum */
template <int d, typename Acc, bool Pairs>
__global__ void __launch_bounds__(RED_THREADS) k_assemble_grad_newton(int64_t nh, const int32_t* __restrict__ gptr,
                                                                       const int32_t* __restrict__ gidx,
                                                                       const double* __restrict__ eg, double* __restrict__ g,
                                                                       double* __restrict__ rhs, double* partials,
                                                                       unsigned* counter, DevScalars* ds, const int32_t* guard)
{
    if (guard && *guard == 0) return;   // every block returns before touching the counter
    double part[1] = {0.0};
    GRID_STRIDE(u, nh)
    {
        double gv[d];
        gather_gradient<d, Acc, Pairs>(u, gptr, gidx, eg, gv);
#pragma unroll
        for (int p = 0; p < d; ++p)
        {
            g[u * d + p] = gv[p];
            rhs[u * d + p] = -gv[p];
            part[0] += gv[p] * gv[p];
        }
    }
    double tot[1];
    if (!grid_sum<1>(part, partials, counter, tot)) return;
    if (threadIdx.x == 0) ds->gg = tot[0];
}

template <typename Acc, bool Pairs>
static void assemble_grad_as(Problem& P)
{
    const unsigned grid = (unsigned)((P.n_handles + 255) / 256);
    switch (P.d)
    {
    case 1: k_assemble_grad<1, Acc, Pairs><<<grid, 256, 0, P.stream>>>(P.n_handles, P.gptr, P.gidx, P.eg, P.g); break;
    case 2: k_assemble_grad<2, Acc, Pairs><<<grid, 256, 0, P.stream>>>(P.n_handles, P.gptr, P.gidx, P.eg, P.g); break;
    default: k_assemble_grad<3, Acc, Pairs><<<grid, 256, 0, P.stream>>>(P.n_handles, P.gptr, P.gidx, P.eg, P.g); break;
    }
}

void launch_assemble_grad(Problem& P, int precision, bool pairs)
{
    if (precision != TAD_PREC_MIXED) assemble_grad_as<double, false>(P);
    else if (pairs) assemble_grad_as<tad::DoubleFloatValue, true>(P);
    else assemble_grad_as<tad::DoubleFloatValue, false>(P);
}

template <typename Acc, bool Pairs>
static void assemble_grad_newton_as(Problem& P)
{
    const unsigned grid = (unsigned)std::min<int64_t>(4 * RED_BLOCKS, std::max<int64_t>(1, (P.n_handles + RED_THREADS - 1) / RED_THREADS));
    switch (P.d)
    {
    case 1: k_assemble_grad_newton<1, Acc, Pairs><<<grid, RED_THREADS, 0, P.stream>>>(P.n_handles, P.gptr, P.gidx, P.eg, P.g, P.rhs,
                                                                                      P.partials, P.counters + 5, P.ds, P.launch_guard); break;
    case 2: k_assemble_grad_newton<2, Acc, Pairs><<<grid, RED_THREADS, 0, P.stream>>>(P.n_handles, P.gptr, P.gidx, P.eg, P.g, P.rhs,
                                                                                      P.partials, P.counters + 5, P.ds, P.launch_guard); break;
    default: k_assemble_grad_newton<3, Acc, Pairs><<<grid, RED_THREADS, 0, P.stream>>>(P.n_handles, P.gptr, P.gidx, P.eg, P.g, P.rhs,
                                                                                       P.partials, P.counters + 5, P.ds, P.launch_guard); break;
    }
}

void launch_assemble_grad_newton(Problem& P, int precision, bool pairs)
{
    if (precision != TAD_PREC_MIXED) assemble_grad_newton_as<double, false>(P);
    else if (pairs) assemble_grad_newton_as<tad::DoubleFloatValue, true>(P);
    else assemble_grad_newton_as<tad::DoubleFloatValue, false>(P);
}

template <int d, typename T>
__global__ void k_assemble_hess(int64_t nb, const int32_t* __restrict__ cptr, const int32_t* __restrict__ cidx,
                                const T* __restrict__ eH, T* __restrict__ H, const int32_t* guard,
                                T* __restrict__ Hs, const int32_t* __restrict__ spos)
{
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= nb || (guard && *guard == 0)) return;
    T acc[d * d];
#pragma unroll
    for (int i = 0; i < d * d; ++i) acc[i] = T(0);
    // contributions in batches of GATHER: the ids, then the blocks, are loaded
    // together (independent loads in flight), then summed in order
    constexpr int GATHER = 4;
    const int32_t q0 = cptr[b], q1 = cptr[b + 1];
    for (int32_t q = q0; q < q1; q += GATHER)
    {
        int32_t c[GATHER];
#pragma unroll
        for (int j = 0; j < GATHER; ++j) c[j] = (q + j < q1) ? cidx[q + j] : 0;
        T v[GATHER][d * d];
#pragma unroll
        for (int j = 0; j < GATHER; ++j)
            if (q + j < q1) tad::load_row<T, d * d>(eH, (int64_t)(c[j] & 0x7fffffff), v[j]);   // one 16-byte load per 2x2 FP32 block
#pragma unroll
        for (int j = 0; j < GATHER; ++j)
        {
            if (q + j >= q1) break;
            if (c[j] < 0)
            {
#pragma unroll
                for (int p = 0; p < d; ++p)
#pragma unroll
                    for (int r = 0; r < d; ++r) acc[p * d + r] += v[j][r * d + p];
            }
            else
            {
#pragma unroll
                for (int i = 0; i < d * d; ++i) acc[i] += v[j][i];
            }
        }
    }
    tad::store_row<T, d * d>(H, b, acc);
    if (Hs) tad::store_row<T, d * d>(Hs, spos[b], acc);   // and its sliced-ELL slot
}

void launch_assemble_hess(Problem& P, int precision)
{
    const unsigned grid = (unsigned)((P.nb + 255) / 256);
    if (P.nb == 0) return;
#define TAD_ASM(D)                                                                                         \
    if (precision == TAD_PREC_MIXED)                                                                       \
        k_assemble_hess<D, float><<<grid, 256, 0, P.stream>>>(P.nb, P.cptr, P.cidx, (const float*)P.eH, (float*)P.H,    \
                                                              P.launch_guard, (float*)P.Hs, P.spos);              \
    else                                                                                                   \
        k_assemble_hess<D, double><<<grid, 256, 0, P.stream>>>(P.nb, P.cptr, P.cidx, (const double*)P.eH, (double*)P.H, \
                                                               P.launch_guard, (double*)P.Hs, P.spos);
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
