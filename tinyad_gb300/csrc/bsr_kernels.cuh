/*
 * bsr_kernels.cuh -- pieces shared by the PCG (solver.cu), the batched PCG
 * (batch.cu) and the AMG hierarchy (amg.cu): precision conversions, BSR
 * block and row loads, inversion of the d x d diagonal blocks and their
 * application to a block row.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "internal.hh"
#include "grid_reduce.cuh"
#include "../../include/tad/Scalar.cuh"

namespace tadlib {

/* conversions between the FP64 vectors and the PCG precision: on this GPU
   float <-> double conversion instructions run on the FP64 pipe, so the FP32
   side uses bit constructions (exact float -> double; double -> nearest
   float through the double-float split) */
template <typename T> __device__ __forceinline__ T from_double(double v);
template <> __device__ __forceinline__ double from_double<double>(double v) { return v; }
template <> __device__ __forceinline__ float from_double<float>(double v) { return (float)tad::DoubleFloatValue(v); }
__device__ __forceinline__ double as_double(double v) { return v; }
__device__ __forceinline__ double as_double(float v) { return tad::DoubleFloat::float_to_double(v); }

/* the d entries of one block row of a vector (one 8-byte load for 2D FP32) */
template <int d, typename T>
__device__ __forceinline__ void load_vec(const T* __restrict__ src, T (&v)[d])
{
    if constexpr (d == 2 && sizeof(T) == 4)
    {
        const float2 q = *reinterpret_cast<const float2*>(src);
        v[0] = q.x; v[1] = q.y;
    }
    else
    {
#pragma unroll
        for (int j = 0; j < d; ++j) v[j] = src[j];
    }
}

/* store the d entries of one block row of a vector (one 8-byte store for 2D FP32) */
template <int d, typename T>
__device__ __forceinline__ void store_vec(T* __restrict__ dst, const T (&v)[d])
{
    if constexpr (d == 2 && sizeof(T) == 4)
        *reinterpret_cast<float2*>(dst) = make_float2(v[0], v[1]);
    else
    {
#pragma unroll
        for (int j = 0; j < d; ++j) dst[j] = v[j];
    }
}

/* one d x d block of H into registers (16-byte vector loads where the
   block size allows) */
template <int d, typename T>
__device__ __forceinline__ void load_block(const T* __restrict__ B, T (&v)[d * d])
{
    if constexpr (d == 2 && sizeof(T) == 4)
    {
        const float4 q = __ldg(reinterpret_cast<const float4*>(B));
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    }
    else if constexpr (d == 2 && sizeof(T) == 8)
    {
        const double2 q0 = __ldg(reinterpret_cast<const double2*>(B));
        const double2 q1 = __ldg(reinterpret_cast<const double2*>(B) + 1);
        v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
    }
    else
    {
#pragma unroll
        for (int i = 0; i < d * d; ++i) v[i] = __ldg(B + i);
    }
}

/* y = (row u of the BSR matrix) z.  The block loop is unrolled four ways
   so four column ids, four blocks and four z gathers are in flight at once
   (the block-at-a-time loop was latency-bound on the bcol -> z dependency). */
template <int d, typename T>
__device__ __forceinline__ void bsr_row_product(const int32_t* __restrict__ bptr, const int32_t* __restrict__ bcol,
                                                const T* __restrict__ H, const T* __restrict__ z, int64_t u, T (&y)[d])
{
#pragma unroll
    for (int i = 0; i < d; ++i) y[i] = T(0);
    int32_t b = bptr[u];
    const int32_t b1 = bptr[u + 1];
    for (; b + 4 <= b1; b += 4)
    {
        int64_t v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = __ldg(bcol + b + k);
        T B[4][d * d], zv[4][d];
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            load_block<d, T>(H + (int64_t)(b + k) * d * d, B[k]);
            load_vec<d, T>(z + v[k] * d, zv[k]);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int i = 0; i < d; ++i)
#pragma unroll
                for (int j = 0; j < d; ++j) y[i] += B[k][i * d + j] * zv[k][j];
    }
    for (; b < b1; ++b)
    {
        const int64_t v = __ldg(bcol + b);
        T B[d * d];
        load_block<d, T>(H + (int64_t)b * d * d, B);
#pragma unroll
        for (int i = 0; i < d; ++i)
#pragma unroll
            for (int j = 0; j < d; ++j) y[i] += B[i * d + j] * z[v * d + j];
    }
}

/* bsr_row_product with the tail predicated: blocks are taken four at a time,
   the last group guarded by the row's end, so a row of 5-7 blocks is two
   rounds of dependent loads (column ids, then blocks and z gathers) instead
   of four, for 48 instead of 32 registers.  The same sums in the same order.
   Used where the kernel has registers to spare (the PCG SpMV: 28.8 -> 27.0 us
   on the 1.64M-face disk, the V-cycle residual); in the post-smoothing's two
   row products it lowered the occupancy and measured slower. */
template <int d, typename T>
__device__ __forceinline__ void bsr_row_product4(const int32_t* __restrict__ bptr, const int32_t* __restrict__ bcol,
                                                const T* __restrict__ H, const T* __restrict__ z, int64_t u, T (&y)[d])
{
#pragma unroll
    for (int i = 0; i < d; ++i) y[i] = T(0);
    const int32_t b1 = bptr[u + 1];
    for (int32_t b = bptr[u]; b < b1; b += 4)
    {
        int64_t v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = b + k < b1 ? __ldg(bcol + b + k) : 0;
        T B[4][d * d], zv[4][d];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (b + k < b1)
            {
                load_block<d, T>(H + (int64_t)(b + k) * d * d, B[k]);
                load_vec<d, T>(z + v[k] * d, zv[k]);
            }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (b + k < b1)
#pragma unroll
                for (int i = 0; i < d; ++i)
#pragma unroll
                    for (int j = 0; j < d; ++j) y[i] += B[k][i * d + j] * zv[k][j];
    }
}

/* y = (row u of the matrix) z from its sliced-ELL copy (Problem::sptr/scol/
   Hs): u's blocks sit at sptr[u/32] + j*32 + u%32, j < the slice's longest
   row (zero blocks beyond u's own).  With rows mapped to consecutive lanes
   (GRID_STRIDE), a warp is one slice: its j-th column ids and blocks are
   contiguous 128- and 32*d*d*sizeof(T)-byte ranges, the block and id loads
   of all j are independent, and no row pointer is loaded.  Blocks are summed
   in the row's order, as bsr_row_product does. */
template <int d, typename T>
__device__ __forceinline__ void sell_row_product(const int32_t* __restrict__ sptr, const int32_t* __restrict__ scol,
                                                 const T* __restrict__ Hs, const T* __restrict__ z, int64_t u, T (&y)[d])
{
#pragma unroll
    for (int i = 0; i < d; ++i) y[i] = T(0);
    const int64_t sl = u >> 5;
    int64_t q = sptr[sl] + (u & 31);
    const int64_t q1 = sptr[sl + 1];
    for (; q + 96 < q1; q += 128)
    {
        int64_t v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = __ldg(scol + q + 32 * k);
        T B[4][d * d], zv[4][d];
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            load_block<d, T>(Hs + (q + 32 * k) * d * d, B[k]);
            load_vec<d, T>(z + v[k] * d, zv[k]);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int i = 0; i < d; ++i)
#pragma unroll
                for (int j = 0; j < d; ++j) y[i] += B[k][i * d + j] * zv[k][j];
    }
    for (; q < q1; q += 32)
    {
        const int64_t v = __ldg(scol + q);
        T B[d * d], zv[d];
        load_block<d, T>(Hs + q * d * d, B);
        load_vec<d, T>(z + v * d, zv);
#pragma unroll
        for (int i = 0; i < d; ++i)
#pragma unroll
            for (int j = 0; j < d; ++j) y[i] += B[i * d + j] * zv[j];
    }
}

/* the sliced-ELL arrays of a problem's H (all null: none, use the BSR form) */
struct SellView
{
    const int32_t* sptr;
    const int32_t* scol;
    const void* Hs;
};

/* The sliced-ELL view of the problem's H when the matrix H handed to a solve
   is that H and the copy exists (other matrices, such as the FP64 copy of a
   mixed solve's completion, have none) */
template <typename T>
inline SellView sell_view(const Problem& P, const T* H)
{
    if (P.Hs && (const void*)H == P.Hs_of) return SellView{P.sptr, P.scol, P.Hs};
    return SellView{nullptr, nullptr, nullptr};
}


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
    T D[d * d];
    load_block<d, T>(dinv + u * d * d, D);
#pragma unroll
    for (int i = 0; i < d; ++i)
    {
        T acc = T(0);
#pragma unroll
        for (int j = 0; j < d; ++j) acc += D[i * d + j] * r[j];
        z[i] = acc;
    }
}

} // namespace tadlib
