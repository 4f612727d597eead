/*
 * bsr_kernels.cuh -- block-Jacobi pieces shared by the PCG (solver.cu) and
 * the AMG hierarchy (amg.cu): inversion of the d x d diagonal blocks and
 * their application to a block row.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "grid_reduce.cuh"

namespace tadlib {

/* ---- block-Jacobi preconditioner: invert (H_uu + w I) ------------------- */
/* inverse of block row u's diagonal block (+ w I) into I; a block that is not
   positive definite (det <= 0 or non-finite) falls back to the inverse of its
   positive diagonal entries (identity where an entry is not positive).  In
   the PCG's precision: FP32 blocks are inverted in FP32 (no FP64
   instructions in the mixed path). */
template <int d, typename T>
__device__ __forceinline__ void diag_block_inverse(const int32_t* __restrict__ diag, const T* __restrict__ H, double w,
                                                   int64_t u, T (&I)[d * d])
{
    T A[d * d];
    const int32_t b = diag[u];
#pragma unroll
    for (int i = 0; i < d * d; ++i) A[i] = b >= 0 ? H[(int64_t)b * d * d + i] : T(0);
#pragma unroll
    for (int i = 0; i < d; ++i) A[i * d + i] += (T)w;
    T det;
    if (d == 1) { det = A[0]; I[0] = T(1) / A[0]; }
    else if (d == 2)
    {
        det = A[0] * A[3] - A[1] * A[2];
        const T id = T(1) / det;
        I[0] = A[3] * id; I[1] = -A[1] * id; I[2] = -A[2] * id; I[3] = A[0] * id;
    }
    else
    {
        const T c00 = A[4] * A[8] - A[5] * A[7], c01 = A[5] * A[6] - A[3] * A[8], c02 = A[3] * A[7] - A[4] * A[6];
        det = A[0] * c00 + A[1] * c01 + A[2] * c02;
        const T id = T(1) / det;
        I[0] = c00 * id; I[3] = c01 * id; I[6] = c02 * id;
        I[1] = (A[2] * A[7] - A[1] * A[8]) * id; I[4] = (A[0] * A[8] - A[2] * A[6]) * id; I[7] = (A[1] * A[6] - A[0] * A[7]) * id;
        I[2] = (A[1] * A[5] - A[2] * A[4]) * id; I[5] = (A[2] * A[3] - A[0] * A[5]) * id; I[8] = (A[0] * A[4] - A[1] * A[3]) * id;
    }
    const bool ok = det > T(0) && isfinite(det);
    if (!ok)
    {
#pragma unroll
        for (int i = 0; i < d; ++i)
#pragma unroll
            for (int j = 0; j < d; ++j)
                I[i * d + j] = (i == j && A[i * d + i] > T(0)) ? T(1) / A[i * d + i] : (i == j ? T(1) : T(0));
    }
}

template <int d, typename T>
__global__ void k_diag_inv(int64_t nh, const int32_t* __restrict__ diag, const T* __restrict__ H, double w, T* __restrict__ dinv)
{
    GRID_STRIDE(u, nh)
    {
        T I[d * d];
        diag_block_inverse<d, T>(diag, H, w, u, I);
#pragma unroll
        for (int i = 0; i < d * d; ++i) dinv[u * d * d + i] = I[i];
    }
}

template <int d, typename T>
__device__ __forceinline__ void apply_dinv(const T* __restrict__ dinv, int64_t u, const T (&r)[d], T (&z)[d])
{
#pragma unroll
    for (int i = 0; i < d; ++i)
    {
        T acc = T(0);
#pragma unroll
        for (int j = 0; j < d; ++j) acc += dinv[u * d * d + i * d + j] * r[j];
        z[i] = acc;
    }
}

} // namespace tadlib
