/*
 * tad_eval_symmetric_dirichlet_tri_noalloc: the total symmetric Dirichlet
 * energy of a triangle parametrisation, computed without allocating any
 * memory.
 *
 * Who needs it: callers that own their device buffers but may not call
 * cudaMalloc themselves or let a library do it -- code that runs while
 * another component is capturing a CUDA graph (an allocation there breaks
 * or invalidates the capture), hosts whose memory pool forbids allocations
 * outside its own allocator, and real-time loops where an allocation's
 * implicit synchronisation is not acceptable.  The regular path
 * (tad_problem_create + tad_eval) allocates its buffers when the problem is
 * created.
 *
 * How: one fused launch evaluates every element's energy (the same
 * tad::SymmetricDirichletTri functor the regular path runs) and reduces the
 * block sums in block order -- the last block to finish adds them up -- so
 * the result is bitwise reproducible.  The reduction scratch (one double per
 * block and an arrival counter) lives in a file-scope __device__ array,
 * g_noalloc_scratch, of 256 B + NOALLOC_MAX_BLOCKS doubles (513 KiB), which
 * every GPU that loads this library holds until the process exits.  Host
 * code may not use the array's name as a device address, so the first call
 * on each device looks its device address up once with
 * cudaGetSymbolAddress (that first call on a device should therefore come
 * before any stream capture).  Each call clears the counter with a memset on
 * the caller's stream; all calls share the one scratch array, so calls that
 * overlap on the GPU (different streams without ordering) race and must be
 * avoided.
 */
#include <mutex>

#include "internal.hh"
#include "../../include/tad/Energies.cuh"

namespace tadlib {

constexpr int NOALLOC_THREADS = 256;
constexpr int64_t NOALLOC_MAX_BLOCKS = 65536;
constexpr int64_t NOALLOC_MAX_FACES = NOALLOC_MAX_BLOCKS * NOALLOC_THREADS;   // 16,777,216
constexpr int NOALLOC_MAX_DEVICES = 64;

/* [0, 4): arrival counter (uint32); [256, ...): per-block partial sums */
static __device__ __align__(256) unsigned char g_noalloc_scratch[256 + NOALLOC_MAX_BLOCKS * sizeof(double)];

static void* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};
static std::mutex g_noalloc_mutex;

__device__ __forceinline__ double warp_sum_na(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(NOALLOC_THREADS) k_symdir_tri_energy_fused(int64_t n, const int32_t* __restrict__ faces,
                                                                            const double* __restrict__ params,
                                                                            const double* __restrict__ x,
                                                                            unsigned char* scratch, double* f_out)
{
    __shared__ double sh[NOALLOC_THREADS / 32];
    __shared__ bool last;
    unsigned* counter = (unsigned*)scratch;
    double* partials = (double*)(scratch + 256);
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double v = 0.0;
    if (e < n)
    {
        tad::PassiveElement<2, 3, double> el{e, x};
        v = tad::SymmetricDirichletTri{faces, params}(el);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    v = warp_sum_na(v);
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0)
    {
        v = lane < NOALLOC_THREADS / 32 ? sh[lane] : 0.0;
        v = warp_sum_na(v);
        if (lane == 0)
        {
            partials[blockIdx.x] = v;
            __threadfence();
            last = (atomicAdd(counter, 1u) == gridDim.x - 1);
        }
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s = 0.0;
    for (int64_t b = threadIdx.x; b < gridDim.x; b += blockDim.x) s += __ldcg(&partials[b]);
    s = warp_sum_na(s);
    if (lane == 0) sh[w] = s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double t = 0.0;
        for (int i = 0; i < NOALLOC_THREADS / 32; ++i) t += sh[i];
        f_out[0] = t;
        *counter = 0u;
    }
}

} // namespace tadlib

using namespace tadlib;

extern "C" TAD_API tad_status tad_eval_symmetric_dirichlet_tri_noalloc(const double* x_d, const int32_t* faces_d,
                                                                      const double* params_d, int64_t n_faces,
                                                                      double* f_d, void* stream)
{
    if (!f_d || (n_faces > 0 && (!x_d || !faces_d || !params_d))) { set_error("NULL argument"); return TAD_ERR_ARG; }
    if (n_faces < 0 || n_faces > NOALLOC_MAX_FACES)
    {
        set_error("n_faces exceeds the no-alloc maximum of 16777216 faces (scratch is a fixed 513 KiB array)");
        return TAD_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0;
    TAD_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) { set_error("device index out of range"); return TAD_ERR_ARG; }
    void* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[dev])
        {
            void* p = nullptr;
            TAD_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
            g_noalloc_ptr[dev] = p;
        }
        scratch = g_noalloc_ptr[dev];
    }
    if (n_faces == 0)
    {
        TAD_CUDA_TRY(cudaMemsetAsync(f_d, 0, sizeof(double), s));
        return TAD_OK;
    }
    TAD_CUDA_TRY(cudaMemsetAsync(scratch, 0, sizeof(unsigned), s));
    const unsigned blocks = (unsigned)((n_faces + NOALLOC_THREADS - 1) / NOALLOC_THREADS);
    k_symdir_tri_energy_fused<<<blocks, NOALLOC_THREADS, 0, s>>>(n_faces, faces_d, params_d, x_d,
                                                                 (unsigned char*)scratch, f_d);
    TAD_CUDA_TRY(cudaGetLastError());
    return TAD_OK;
}
