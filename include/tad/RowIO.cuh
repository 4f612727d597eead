/*
 * tad/RowIO.cuh -- vectorised access to row e of a row-major [n][W] device
 * array (element outputs, element blocks, BSR blocks).
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tad {

/* Row e of a row-major [n][W] array of T: 16-byte vector accesses when the
   row size is a multiple of 16 bytes and the array is 16-byte aligned (a
   term's slice of the shared element buffers need not be), scalar ones
   otherwise.  Fewer memory instructions per element keep the element
   kernels off the load/store queue limit. */
template <typename T, int W>
__device__ __forceinline__ void store_row(T* base, int64_t e, const T (&v)[W])
{
    T* dst = base + e * W;
    if constexpr ((W * sizeof(T)) % 16 == 0 && (sizeof(T) == 4 || sizeof(T) == 8))
    {
        if ((reinterpret_cast<uintptr_t>(base) & 15) == 0)
        {
            if constexpr (sizeof(T) == 4)
            {
#pragma unroll
                for (int i = 0; i < W / 4; ++i)
                    reinterpret_cast<float4*>(dst)[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
            }
            else
            {
#pragma unroll
                for (int i = 0; i < W / 2; ++i) reinterpret_cast<double2*>(dst)[i] = make_double2(v[2 * i], v[2 * i + 1]);
            }
            return;
        }
    }
#pragma unroll
    for (int i = 0; i < W; ++i) dst[i] = v[i];
}
template <typename T, int W>
__device__ __forceinline__ void load_row(const T* base, int64_t e, T (&v)[W])
{
    const T* src = base + e * W;
    if constexpr ((W * sizeof(T)) % 16 == 0 && (sizeof(T) == 4 || sizeof(T) == 8))
    {
        if ((reinterpret_cast<uintptr_t>(base) & 15) == 0)
        {
            if constexpr (sizeof(T) == 4)
            {
#pragma unroll
                for (int i = 0; i < W / 4; ++i)
                {
                    const float4 q = reinterpret_cast<const float4*>(src)[i];
                    v[4 * i] = q.x; v[4 * i + 1] = q.y; v[4 * i + 2] = q.z; v[4 * i + 3] = q.w;
                }
            }
            else
            {
#pragma unroll
                for (int i = 0; i < W / 2; ++i)
                {
                    const double2 q = reinterpret_cast<const double2*>(src)[i];
                    v[2 * i] = q.x; v[2 * i + 1] = q.y;
                }
            }
            return;
        }
    }
#pragma unroll
    for (int i = 0; i < W; ++i) v[i] = src[i];
}

} // namespace tad
