/*
 * grid_reduce.cuh -- deterministic grid-wide reductions shared by the
 * solver kernels: warp shuffles, a fixed-order block sum, and the "last
 * block" grid sum (block partials, then the last block to arrive adds them
 * in block order; one atomic counter, no spinning, no float atomics).
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tadlib {

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

/* fixed-order sum of NV values over the block; results valid in thread 0 */
template <int NV>
__device__ __forceinline__ void block_sum_n(double (&v)[NV], double (*sh)[32])
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = warp_sum_d(v[i]);
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < NV; ++i) sh[i][w] = v[i];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i)
    {
        v[i] = 0.0;
        if (w == 0)
        {
            v[i] = (lane < (int)(blockDim.x >> 5)) ? sh[i][lane] : 0.0;
            v[i] = warp_sum_d(v[i]);
        }
    }
    __syncthreads();
}

/* Grid-wide reduction of NV values: block partials, then the last block to
   arrive sums them in block order.  Returns true in the last block, with the
   totals in tot (all threads). */
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double* partials, unsigned* counter, double (&tot)[NV])
{
    __shared__ double sh[NV][32];
    __shared__ bool last;
    __shared__ double res[NV];
    block_sum_n<NV>(v, sh);
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int i = 0; i < NV; ++i) partials[i * gridDim.x + blockIdx.x] = v[i];
        __threadfence();
        const unsigned t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i)
    {
        s[i] = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s[i] += __ldcg(&partials[i * gridDim.x + b]);
    }
    block_sum_n<NV>(s, sh);
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int i = 0; i < NV; ++i) res[i] = s[i];
        *counter = 0u;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) tot[i] = res[i];
    return true;
}

#define GRID_STRIDE(i, n) for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

} // namespace tadlib
