/*
 * Batched Projected Newton: many independent meshes of uneven sizes solved
 * together.  No reference counterpart (TinyAD solves one ScalarFunction at a
 * time); each mesh follows the single-problem algorithm with the block-Jacobi
 * preconditioner (settings.preconditioner = 0: no AMG restart) and at most
 * 16 Armijo trials.
 *
 * Layout: the meshes are concatenated into one block-diagonal problem
 * (handles offset per mesh), so the element kernels, the assembly and the
 * BSR SpMV run unchanged -- one launch per stage for all meshes.  Everything
 * that is per mesh -- energies, dot products, PCG alpha/beta/convergence,
 * the Armijo choice and step -- is computed over "chunks": contiguous ranges
 * of block rows (or elements) that each belong to one mesh.  A kernel walks
 * the chunk list with a fixed grid (grid-stride over chunks); the last
 * chunk of a mesh to finish sums that mesh's chunk partials in chunk order,
 * so every per-mesh reduction is deterministic.
 *
 * One Newton iteration (elements -> f -> assembly, only when some mesh did
 * not take the previous full step -> PCG, each mesh stopping at its own
 * tolerance, all iterations in one persistent launch whose chunk list
 * follows the meshes still iterating -> the full step, evaluated by the
 * element kernels and assembly at x + d, which are the next iteration's
 * derivatives -> batches of 8 and 7 energy-only trials while some mesh has
 * not accepted one -> per-mesh step) has a fixed launch sequence and is
 * captured once as a CUDA graph; the host replays one graph per iteration.
 * Trial kernels after every mesh has accepted a step return at once (a
 * device counter).
 * A small autotuner times candidate chunk sizes / block sizes on the batch
 * itself and keeps the fastest.
 */
#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "internal.hh"
#include "bsr_kernels.cuh"

namespace tadlib {

struct Chunk
{
    int32_t mesh, begin, end;
};

struct BatchScalars
{
    double* f;        // [m] energy
    double* ftr;      // [m][16] trial energies
    double* gg;       // [m]
    double* dg;       // [m]
    double* rz;       // [m]
    double* bb;
    double* tol2;
    double* alpha;
    double* beta;
    double* rr;
    int32_t* done;    // [m]
    int32_t* iters;   // [m]
    int32_t* choice;  // [m] accepted trial, -1 none, -3 none and stalled in this iteration
    double* step;     // [m]
    int32_t* searching;   // meshes without an accepted trial after the last selection
    int32_t* stalled;     // [m] no trial step passed the Armijo test: x stays, and so would every later
                          // iteration's result; the mesh is left out of the PCG and the line search
                          // until the next solve call
    int32_t* need_eval;   // meshes that rejected the full step in the last iteration (0: the
                          // derivatives assembled at x + d are those of every mesh's new x)
    double* f_start;      // [m] energy at the start of the last iteration (the history)
    double* pap;          // [m] p.Ap of the persistent PCG's last SpMV phase
};

constexpr int LS_TRIALS = 16;

__device__ __forceinline__ double bw_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int NV>
__device__ __forceinline__ void bblock_sum(double (&v)[NV], double (*sh)[32])
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = bw_sum(v[i]);
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
            v[i] = lane < (int)(blockDim.x >> 5) ? sh[i][lane] : 0.0;
            v[i] = bw_sum(v[i]);
        }
    }
    __syncthreads();
}

/* Block-level chunk reduction + per-mesh completion.  Returns true in the
   block that completed mesh m (totals in tot, all threads). */
template <int NV>
__device__ bool seg_finish(int ci, int m, double (&v)[NV], double* partials, int n_chunks, unsigned* counters,
                           const int32_t* mc_begin, const int32_t* mc_end, double (&tot)[NV])
{
    __shared__ double sh[NV][32];
    __shared__ bool last;
    __shared__ double res[NV];
    bblock_sum<NV>(v, sh);
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int i = 0; i < NV; ++i) partials[(int64_t)i * n_chunks + ci] = v[i];
        __threadfence();
        const unsigned cnt = (unsigned)(mc_end[m] - mc_begin[m]);
        last = atomicAdd(&counters[m], 1u) == cnt - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i)
    {
        s[i] = 0.0;
        for (int c = mc_begin[m] + threadIdx.x; c < mc_end[m]; c += blockDim.x)
            s[i] += __ldcg(&partials[(int64_t)i * n_chunks + c]);
    }
    bblock_sum<NV>(s, sh);
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int i = 0; i < NV; ++i) res[i] = s[i];
        counters[m] = 0u;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) tot[i] = res[i];
    return true;
}

/* per-mesh sums of element-energy rows: out[m * stride_out + row] */
__global__ void k_b_reduce_rows(const Chunk* ch, int n_chunks, const int32_t* mcb, const int32_t* mce, const double* ef,
                                int64_t row_stride, double* partials, unsigned* counters, double* out, int out_stride,
                                const int32_t* active = nullptr)
{
    // active: as for the line-search element kernels, 0 = nothing to sum (every block
    // returns before touching the segment counters)
    if (active && *active == 0) return;
    const int row = blockIdx.y;
    for (int ci = blockIdx.x; ci < n_chunks; ci += gridDim.x)
    {
        const Chunk c = ch[ci];
        double v[1] = {0.0};
        for (int i = c.begin + threadIdx.x; i < c.end; i += blockDim.x) v[0] += ef[row * row_stride + i];
        double tot[1];
        if (seg_finish<1>(ci, c.mesh, v, partials + (int64_t)row * n_chunks, n_chunks, counters + row * 4096, mcb, mce, tot) &&
            threadIdx.x == 0)
            out[(int64_t)c.mesh * out_stride + row] = tot[0];
    }
}

/* per-mesh a.b over block-row chunks (d values per row) */
template <int d>
__global__ void k_b_dot(const Chunk* ch, int n_chunks, const int32_t* mcb, const int32_t* mce, const double* a,
                        const double* b, double* partials, unsigned* counters, double* out)
{
    for (int ci = blockIdx.x; ci < n_chunks; ci += gridDim.x)
    {
        const Chunk c = ch[ci];
        double v[1] = {0.0};
        for (int64_t i = (int64_t)c.begin * d + threadIdx.x; i < (int64_t)c.end * d; i += blockDim.x) v[0] += a[i] * b[i];
        double tot[1];
        if (seg_finish<1>(ci, c.mesh, v, partials, n_chunks, counters, mcb, mce, tot) && threadIdx.x == 0)
            out[c.mesh] = tot[0];
    }
}

/* exclusive prefix sum over the block (one value per thread); total: the sum */
template <typename V>
__device__ __forceinline__ V block_exclusive_scan(V v, V* warp_tot, V& total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    V inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const V u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0)
    {
        V x = lane < nw ? warp_tot[lane] : V(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const V u = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += u;
        }
        warp_tot[lane] = x;   // inclusive over warps
    }
    __syncthreads();
    const V before = w == 0 ? V(0) : warp_tot[w - 1];
    total = warp_tot[nw - 1];
    __syncthreads();
    return before + inc - v;
}

/* per mesh: x = 0, r = b, z = D^-1 r with the diagonal blocks inverted here
   in the PCG precision (D^-1 stored), p = Ap = 0, beta = 0 (the first fused
   SpMV then forms p = z, Ap = H z); rz, bb, tol2, iters = 0, done = (b == 0) */
template <int d, typename T>
__global__ void k_b_pcg_init(const Chunk* ch, int n_chunks, const int32_t* mcb, const int32_t* mce, const double* b,
                             const int32_t* __restrict__ diag, const T* __restrict__ H, T* x, T* r, T* z, T* p, T* Ap,
                             T* dinv, double* partials, unsigned* counters, BatchScalars S, double rel_tol)
{
    for (int ci = blockIdx.x; ci < n_chunks; ci += gridDim.x)
    {
        const Chunk c = ch[ci];
        T acc_rz = T(0), acc_bb = T(0);
        for (int64_t u = c.begin + threadIdx.x; u < c.end; u += blockDim.x)
        {
            T rv[d], I[d * d];
            diag_block_inverse<d, T>(diag, H, 0.0, u, I);
#pragma unroll
            for (int i = 0; i < d; ++i) { rv[i] = from_double<T>(b[u * d + i]); x[u * d + i] = T(0); r[u * d + i] = rv[i]; }
#pragma unroll
            for (int i = 0; i < d; ++i)
            {
                T acc = T(0);
#pragma unroll
                for (int j = 0; j < d; ++j) { acc += I[i * d + j] * rv[j]; dinv[u * d * d + i * d + j] = I[i * d + j]; }
                z[u * d + i] = acc;
                p[u * d + i] = T(0);
                Ap[u * d + i] = T(0);
                acc_rz += rv[i] * acc;
                acc_bb += rv[i] * rv[i];
            }
        }
        double v[2] = {as_double(acc_rz), as_double(acc_bb)}, tot[2];
        if (seg_finish<2>(ci, c.mesh, v, partials, n_chunks, counters, mcb, mce, tot) && threadIdx.x == 0)
        {
            const int m = c.mesh;
            S.rz[m] = tot[0];
            S.bb[m] = tot[1];
            S.rr[m] = tot[1];
            S.tol2[m] = rel_tol * rel_tol * tot[1];
            S.iters[m] = 0;
            S.beta[m] = 0.0;
            S.done[m] = (tot[1] == 0.0 || S.stalled[m]) ? 1 : 0;
        }
    }
}

/* ---- the PCG stage as one persistent launch ------------------------------
   All PCG iterations of a batched Newton iteration run in one launch of a
   grid that fits on the GPU at once (cooperative launch where the capture
   allows it).  Each iteration is two phases separated by grid barriers:
     SpMV    Ap = H z + beta Ap, p = z + beta p, p.Ap -> alpha (per mesh)
     update  x += alpha p, r -= alpha Ap, z = D^-1 r, r.z and r.r -> beta,
             the stop test (per mesh)
   Every block derives the same chunk list from the meshes still iterating
   at the start of the iteration (their rows cut into chunks of
   C = max(min_rows, ceil(R / 4G)) rows), so the work of the remaining
   meshes spreads over the whole grid without a rebuild kernel; blocks take
   chunks from a per-phase counter, so the blocks that drew short chunks
   take more (a static assignment left the grid waiting at the barriers
   for its slowest blocks).  Per-mesh
   sums: the last chunk of a mesh to finish adds that mesh's chunk partials
   in chunk order (deterministic).  Rows move between blocks as meshes
   finish; a phase reads what other SMs wrote in the phase before with
   ordinary loads, ordered by the barrier: its waiting thread's GPU-scope
   fence after the generation changes, then __syncthreads, as in a
   cooperative grid synchronisation.  The barriers wait a bounded time: a wait
   that gives up sets bit 8 of the device error word (TAD_ERR_TIMEOUT) and
   every block leaves the loop at its next barrier. */
constexpr int PB_THREADS = 256;                 // block size of the launch bound (8 blocks per SM: full occupancy); the launch uses the batch's
                                                // threads per block and its pb_per_sm blocks per SM (autotuned)
constexpr long long PB_SPIN_LIMIT = 1LL << 23;   // ~2-4 s of polling with __nanosleep(256)

struct GridBarrier
{
    unsigned* count;   // arrivals of the current barrier
    unsigned* gen;     // barrier generation (on another 128-byte line than count: the
                       // waiting blocks poll it while the others still arrive)
    int32_t* err;      // the problem's device error word
};

/* all blocks of the grid; false if this or another block's wait gave up */
__device__ __forceinline__ bool grid_barrier(const GridBarrier& gb)
{
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        volatile unsigned* vgen = gb.gen;
        const unsigned g = *vgen;
        __threadfence();
        int ok = 0;
        if (atomicAdd(gb.count, 1u) == gridDim.x - 1)
        {
            *gb.count = 0u;
            __threadfence();
            atomicAdd(gb.gen, 1u);
            ok = 1;
        }
        else
        {
            for (long long k = 0; k < PB_SPIN_LIMIT; ++k)
            {
                if (*vgen != g) { ok = 1; break; }
                if (*(volatile int32_t*)gb.err & 8) break;
                __nanosleep(256);
            }
            if (!ok) atomicOr(gb.err, 8);
        }
        __threadfence();
        ok_s = ok && !(*(volatile int32_t*)gb.err & 8);
    }
    __syncthreads();
    return ok_s != 0;
}

/* the chunk list of the meshes still iterating, in shared memory: start[m]
   = first chunk of mesh m (start[n_meshes] = total), chunk size C */
__device__ __forceinline__ void pb_chunk_list(int n_meshes, const int64_t* __restrict__ row_off, const int32_t* done,
                                              int min_rows, int32_t* start, long long& C_out)
{
    __shared__ long long red_ll[32];
    __shared__ int red_i[32];
    __shared__ long long C_s;
    const int per = (n_meshes + blockDim.x - 1) / blockDim.x;
    const int m0 = min(n_meshes, (int)threadIdx.x * per), m1 = min(n_meshes, m0 + per);
    long long rows = 0;
    for (int m = m0; m < m1; ++m)
        if (!*(volatile const int32_t*)&done[m]) rows += row_off[m + 1] - row_off[m];
    long long R;
    (void)block_exclusive_scan<long long>(rows, red_ll, R);
    if (threadIdx.x == 0) C_s = max((long long)min_rows, (R + 4LL * gridDim.x - 1) / (4LL * gridDim.x));
    __syncthreads();
    const long long C = C_s;
    int cnt = 0;
    for (int m = m0; m < m1; ++m)
        if (!*(volatile const int32_t*)&done[m]) cnt += (int)((row_off[m + 1] - row_off[m] + C - 1) / C);
    int total;
    int off = block_exclusive_scan<int>(cnt, red_i, total);
    for (int m = m0; m < m1; ++m)
    {
        start[m] = off;
        if (!*(volatile const int32_t*)&done[m]) off += (int)((row_off[m + 1] - row_off[m] + C - 1) / C);
    }
    if (threadIdx.x == 0) start[n_meshes] = total;
    __syncthreads();
    C_out = C;
}

/* mesh of chunk c: the last m with start[m] <= c (meshes without chunks have start[m] == start[m+1]) */
__device__ __forceinline__ int pb_mesh_of(const int32_t* start, int n_meshes, int c)
{
    int lo = 0, hi = n_meshes;   // start[lo] <= c < start[hi]
    while (hi - lo > 1)
    {
        const int mid = (lo + hi) >> 1;
        if (start[mid] <= c) lo = mid;
        else hi = mid;
    }
    return lo;
}

/* the block's share of one per-mesh sum: NV block partials into partials[i * stride + c]; the last
   chunk of mesh m to arrive (cnt chunks) sums them in chunk order into tot (all threads) */
template <int NV>
__device__ __forceinline__ bool pb_finish(int c, int c0, int cnt, int m, double (&v)[NV], double* partials, int stride,
                                          unsigned* counters, double (&tot)[NV])
{
    __shared__ double sh[NV][32];
    __shared__ bool last;
    __shared__ double res[NV];
    bblock_sum<NV>(v, sh);
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int i = 0; i < NV; ++i) partials[(int64_t)i * stride + c] = v[i];
        __threadfence();
        last = atomicAdd(&counters[m], 1u) == (unsigned)cnt - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s2[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i)
    {
        s2[i] = 0.0;
        for (int k = c0 + threadIdx.x; k < c0 + cnt; k += blockDim.x) s2[i] += __ldcg(&partials[(int64_t)i * stride + k]);
    }
    bblock_sum<NV>(s2, sh);
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int i = 0; i < NV; ++i) res[i] = s2[i];
        counters[m] = 0u;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) tot[i] = res[i];
    return true;
}

/* the block's next chunk of the phase whose counter is ctr (all threads) */
__device__ __forceinline__ int pb_next_chunk(unsigned* ctr)
{
    __shared__ int c_s;
    __syncthreads();   // the previous chunk's readers of c_s are done
    if (threadIdx.x == 0) c_s = (int)atomicAdd(ctr, 1u);
    __syncthreads();
    return c_s;
}

template <int d, typename T>
__global__ void __launch_bounds__(PB_THREADS, sizeof(T) == 4 ? 8 : 4) k_b_pcg_persistent(int n_meshes, const int64_t* __restrict__ row_off,
                                                                 int min_rows, const int32_t* __restrict__ bptr,
                                                                 const int32_t* __restrict__ bcol, const T* __restrict__ H,
                                                                 T* x, T* r, T* z, T* p, T* Ap, const T* __restrict__ dinv,
                                                                 double* partials, int stride, unsigned* counters,
                                                                 BatchScalars S, int max_iters, GridBarrier gb,
                                                                 unsigned* work)
{
    // work[4]: chunk counters of the two phases of even and odd iterations;
    // zero at launch; those of the next iteration are cleared during the
    // update phase (their last users finished before the previous barrier)
    extern __shared__ int32_t start[];   // n_meshes + 1
    for (int it = 0; it < max_iters; ++it)
    {
        long long C;
        pb_chunk_list(n_meshes, row_off, S.done, min_rows, start, C);
        const int n_chunks = start[n_meshes];
        if (n_chunks == 0) break;   // every mesh is done (the same decision in every block)
        unsigned* ctr = work + 2 * (it & 1);
        // SpMV phase
        for (int c = pb_next_chunk(ctr); c < n_chunks; c = pb_next_chunk(ctr))
        {
            const int m = pb_mesh_of(start, n_meshes, c);
            const int c0 = start[m], cnt = start[m + 1] - c0;
            const int64_t b0 = row_off[m] + (int64_t)(c - c0) * C;
            const int64_t b1 = min((long long)row_off[m + 1], (long long)(b0 + C));
            const T beta = from_double<T>(S.beta[m]);
            T part = T(0);
            for (int64_t u = b0 + threadIdx.x; u < b1; u += blockDim.x)
            {
                T y[d];
                bsr_row_product<d, T>(bptr, bcol, H, z, u, y);
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
            // done flags change only in the update phase: blocks still building this
            // iteration's chunk list read them, so a breakdown is recorded in pap and
            // acted on by the update's finisher (alpha = 0 leaves x and r as they are)
            double v[1] = {as_double(part)}, tot[1];
            if (pb_finish<1>(c, c0, cnt, m, v, partials, stride, counters, tot) && threadIdx.x == 0)
            {
                S.pap[m] = tot[0];
                S.alpha[m] = (tot[0] > 0.0 && isfinite(tot[0])) ? S.rz[m] / tot[0] : 0.0;
            }
        }
        if (!grid_barrier(gb)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0)
        {
            work[2 * ((it + 1) & 1)] = 0u;
            work[2 * ((it + 1) & 1) + 1] = 0u;
        }
        // update phase
        for (int c = pb_next_chunk(ctr + 1); c < n_chunks; c = pb_next_chunk(ctr + 1))
        {
            const int m = pb_mesh_of(start, n_meshes, c);
            const int c0 = start[m], cnt = start[m + 1] - c0;
            const int64_t b0 = row_off[m] + (int64_t)(c - c0) * C;
            const int64_t b1 = min((long long)row_off[m + 1], (long long)(b0 + C));
            const T alpha = from_double<T>(S.alpha[m]);
            T acc_rz = T(0), acc_rr = T(0);
            for (int64_t u = b0 + threadIdx.x; u < b1; u += blockDim.x)
            {
                T rv[d], zv[d];
#pragma unroll
                for (int i = 0; i < d; ++i)
                {
                    x[u * d + i] += alpha * p[u * d + i];
                    rv[i] = r[u * d + i] - alpha * Ap[u * d + i];
                    r[u * d + i] = rv[i];
                }
                apply_dinv<d, T>(dinv, u, rv, zv);
#pragma unroll
                for (int i = 0; i < d; ++i)
                {
                    z[u * d + i] = zv[i];
                    acc_rz += rv[i] * zv[i];
                    acc_rr += rv[i] * rv[i];
                }
            }
            double v[2] = {as_double(acc_rz), as_double(acc_rr)}, tot[2];
            if (pb_finish<2>(c, c0, cnt, m, v, partials, stride, counters, tot) && threadIdx.x == 0)
            {
                const double pap = S.pap[m];
                if (!(pap > 0.0) || !isfinite(pap)) { S.done[m] = 1; continue; }   // non-positive curvature
                S.beta[m] = tot[0] / S.rz[m];
                S.rz[m] = tot[0];
                S.rr[m] = tot[1];
                S.iters[m] += 1;
                if (tot[1] <= S.tol2[m] || S.iters[m] >= max_iters || !isfinite(tot[1])) S.done[m] = 1;
            }
        }
        if (!grid_barrier(gb)) return;
    }
}

template <typename T>
__global__ void k_b_to_double(int64_t n, const T* a, double* out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = as_double(a[i]);
}

/* per-mesh Armijo choice among trials [t0, t0 + nt) (LineSearch.hh:14-24);
   a mesh left without a step after the last trial is stalled (the single
   problem's Newton loop stops there) */
__global__ void k_b_ls_select(int n_meshes, int t0, int nt, const double* steps, double c_armijo, BatchScalars S)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n_meshes) return;
    if (t0 == 0) S.choice[m] = -1;
    if (S.choice[m] >= 0 || S.stalled[m]) return;
    for (int j = 0; j < nt; ++j)
    {
        const double fn = S.ftr[m * LS_TRIALS + t0 + j];
        if (fn <= S.f[m] + c_armijo * steps[t0 + j] * S.dg[m])
        {
            S.choice[m] = t0 + j;
            S.step[m] = steps[t0 + j];
            return;
        }
    }
    if (t0 + nt >= LS_TRIALS) { S.stalled[m] = 1; S.choice[m] = -3; }
    else atomicAdd(S.searching, 1);   // the later trial launches return at once when none search
}

template <int d>
__global__ void k_b_axpy(const Chunk* ch, int n_chunks, double* x, const double* dx, BatchScalars S, int apply_all)
{
    for (int ci = blockIdx.x; ci < n_chunks; ci += gridDim.x)
    {
        const Chunk c = ch[ci];
        if (S.choice[c.mesh] < 0) continue;
        const double s = S.step[c.mesh];
        for (int64_t i = (int64_t)c.begin * d + threadIdx.x; i < (int64_t)c.end * d; i += blockDim.x) x[i] += s * dx[i];
    }
}

/* energy of the next iteration's x: the full step's (trial 0, evaluated with
   the derivatives at x + d) for the meshes that took it, and for meshes
   stalled before this iteration (their d is 0, so trial 0 is x itself); a
   mesh that stalled in this iteration (choice -3) keeps f(x), since its
   trial 0 was the rejected point; the others are evaluated afresh
   (need_eval) */
__global__ void k_b_adopt_f(int n_meshes, BatchScalars S)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n_meshes) return;
    if (S.choice[m] == 0 || (S.stalled[m] && S.choice[m] != -3)) S.f[m] = S.ftr[m * LS_TRIALS];
}

template <int d>
__global__ void k_b_add(int64_t n, const double* __restrict__ x, const double* __restrict__ dx, double* __restrict__ xt)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        xt[i] = x[i] + dx[i];
}

/* line-search trial energies of meshes that have not accepted a step yet are
   computed for all meshes (one launch); k_b_ls_select ignores the rest */

struct Batch
{
    tad_problem* P = nullptr;
    int n_meshes = 0;
    std::vector<int64_t> vert_off;           // per mesh handle offset (n_meshes + 1)
    std::vector<std::vector<int64_t>> elem_cnt; // per term, per mesh element counts (built while adding)
    int chunk_rows = 1024, threads = 256, grid = 0;   // grid: 4 blocks per SM, set when the batch is prepared
    // device
    Chunk *vch = nullptr, *ech = nullptr;
    int n_vch = 0, n_ech = 0;
    int32_t *vmcb = nullptr, *vmce = nullptr, *emcb = nullptr, *emce = nullptr;
    // per-mesh row offsets (the persistent PCG's chunk lists); chunk capacity
    // of the persistent PCG (2 x its grid + n_meshes)
    int64_t* row_off = nullptr;
    int pch_cap = 0;
    double* partials = nullptr;
    unsigned* counters = nullptr;   // [LS_TRIALS * 4096]
    double* scal = nullptr;
    int32_t* iscal = nullptr;
    BatchScalars S{};
    double* steps = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_iters = 0;
    double* fh = nullptr;           // pinned [n_meshes]
    double* x = nullptr;            // device state
    double* xt = nullptr;           // x + d, where the full step's derivatives are evaluated
    int pcg_iters = 64;
    double pcg_tol = 1e-2;
    int sms = 0;                    // the device's SM count
    int pb_per_sm = 8;              // blocks per SM of the persistent PCG (at most what fits)
    bool cooperative = false;       // cooperative launches can be captured (the persistent PCG's co-residency guarantee)
    unsigned* bar = nullptr;        // [64]: grid-barrier arrival count [0], generation [32], chunk counters [48..51]
};

static std::vector<Chunk> make_chunks(const std::vector<int64_t>& off, int rows, std::vector<int32_t>& mcb, std::vector<int32_t>& mce)
{
    std::vector<Chunk> out;
    const int nm = (int)off.size() - 1;
    mcb.assign(nm, 0);
    mce.assign(nm, 0);
    for (int m = 0; m < nm; ++m)
    {
        mcb[m] = (int32_t)out.size();
        for (int64_t b = off[m]; b < off[m + 1]; b += rows)
            out.push_back({m, (int32_t)b, (int32_t)std::min<int64_t>(off[m + 1], b + rows)});
        mce[m] = (int32_t)out.size();
    }
    return out;
}

static tad_status batch_fail(tad_status s, const char* m) { set_error(m); return s; }

template <typename X>
static cudaError_t upload(X** d, const std::vector<X>& h)
{
    cudaError_t e = cudaMalloc((void**)d, std::max<size_t>(h.size(), 1) * sizeof(X));
    if (e != cudaSuccess) return e;
    return h.empty() ? cudaSuccess : cudaMemcpy(*d, h.data(), h.size() * sizeof(X), cudaMemcpyHostToDevice);
}

static tad_status batch_setup_chunks(Batch& B)
{
    Problem& P = *B.P;
    if (B.vch) { cudaFree(B.vch); cudaFree(B.ech); cudaFree(B.vmcb); cudaFree(B.vmce); cudaFree(B.emcb); cudaFree(B.emce); }
    std::vector<int32_t> vmcb, vmce, emcb, emce;
    std::vector<Chunk> vch = make_chunks(B.vert_off, B.chunk_rows, vmcb, vmce);
    // element chunks: per mesh, over every term (elements of a mesh are contiguous within a term)
    std::vector<Chunk> ech;
    emcb.assign(B.n_meshes, 0);
    emce.assign(B.n_meshes, 0);
    for (int m = 0; m < B.n_meshes; ++m)
    {
        emcb[m] = (int32_t)ech.size();
        for (size_t t = 0; t < P.terms.size(); ++t)
        {
            int64_t beg = P.terms[t].elem_off;
            for (int mm = 0; mm < m; ++mm) beg += B.elem_cnt[t][mm];
            const int64_t end = beg + B.elem_cnt[t][m];
            for (int64_t b = beg; b < end; b += 4 * B.chunk_rows)
                ech.push_back({m, (int32_t)b, (int32_t)std::min<int64_t>(end, b + 4 * B.chunk_rows)});
        }
        emce[m] = (int32_t)ech.size();
        if (emce[m] == emcb[m]) ech.push_back({m, 0, 0}), emce[m] = (int32_t)ech.size();
    }
    B.n_vch = (int)vch.size();
    B.n_ech = (int)ech.size();
    TAD_CUDA_TRY(upload(&B.vch, vch));
    TAD_CUDA_TRY(upload(&B.ech, ech));
    TAD_CUDA_TRY(upload(&B.vmcb, vmcb));
    TAD_CUDA_TRY(upload(&B.vmce, vmce));
    TAD_CUDA_TRY(upload(&B.emcb, emcb));
    TAD_CUDA_TRY(upload(&B.emce, emce));
    B.pch_cap = 4 * B.sms * 16 + B.n_meshes;   // the persistent PCG's chunks: at most 4 per block + n_meshes
    if (!B.row_off) TAD_CUDA_TRY(upload(&B.row_off, B.vert_off));
    if (B.partials) cudaFree(B.partials);
    const size_t n_part = std::max<size_t>((size_t)std::max(B.n_vch, B.n_ech) * LS_TRIALS, (size_t)B.pch_cap) * 2;
    TAD_CUDA_TRY(cudaMalloc(&B.partials, n_part * sizeof(double)));
    return TAD_OK;
}

/* record one batched Newton iteration on the problem's stream (captured) */
template <int d, typename T>
static tad_status record_iteration(Batch& B, int prec, double eps)
{
    Problem& P = *B.P;
    cudaStream_t s = P.stream;
    const int G = B.grid, TH = B.threads;
    const int64_t n = P.n_vars;
    T* H = (T*)P.H;
    T *r, *z, *p, *Ap, *xs, *dinv;
    if (prec == TAD_PREC_MIXED) { r = (T*)P.r32; z = (T*)P.z32; p = (T*)P.p32; Ap = (T*)P.Ap32; xs = (T*)P.dx32; dinv = (T*)P.dinv32; }
    else { r = (T*)P.r; z = (T*)P.z; p = (T*)P.p; Ap = (T*)P.Ap; xs = (T*)P.dx; dinv = (T*)P.dinv; }
    // 1. element Hessians at x (all meshes, one launch per term), f per mesh,
    // assembly of g, rhs = -g and H -- only when some mesh did not take the
    // previous iteration's full step (or a solve call starts): otherwise the
    // derivatives assembled at that step's x + d are current
    P.launch_guard = B.S.need_eval;
    tad_status st = eval_elements(P, TAD_MODE_HESSIAN_PROJ, B.x, eps, prec);
    if (st == TAD_OK)
    {
        k_b_reduce_rows<<<dim3(G, 1), TH, 0, s>>>(B.ech, B.n_ech, B.emcb, B.emce, P.ef, P.n_elem_total, B.partials,
                                                  B.counters, B.S.f, 1, B.S.need_eval);
        launch_assemble_grad_newton(P, prec, prec == TAD_PREC_MIXED);
        launch_assemble_hess(P, prec);
    }
    P.launch_guard = nullptr;
    if (st != TAD_OK) return st;
    TAD_CUDA_TRY(cudaMemcpyAsync(B.S.f_start, B.S.f, (size_t)B.n_meshes * sizeof(double), cudaMemcpyDeviceToDevice, s));
    // 2. PCG, per-mesh tolerance: the init (per-mesh scalars, the inverted
    // diagonal blocks), then every iteration in one persistent launch
    k_b_pcg_init<d, T><<<G, TH, 0, s>>>(B.vch, B.n_vch, B.vmcb, B.vmce, P.rhs, P.diag, H, xs, r, z, p, Ap, dinv,
                                        B.partials, B.counters, B.S, B.pcg_tol);
    {
        int per_sm = 0;
        const size_t smem = (size_t)(B.n_meshes + 1) * sizeof(int32_t);
        const int pth = std::min(TH, PB_THREADS);
        TAD_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_b_pcg_persistent<d, T>, pth, smem));
        const int Gp = std::max(1, B.sms * std::min(std::max(per_sm, 1), B.pb_per_sm));
        GridBarrier gb{B.bar, B.bar + 32, P.err};
        // a barrier count left over by a launch that gave up starts from zero
        // again; the chunk counters (bar[48..51]) start at zero
        TAD_CUDA_TRY(cudaMemsetAsync(B.bar, 0, sizeof(unsigned), s));
        TAD_CUDA_TRY(cudaMemsetAsync(B.bar + 48, 0, 4 * sizeof(unsigned), s));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)Gp);
        cfg.blockDim = dim3(pth);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = s;
        cudaLaunchAttribute attr;
        attr.id = cudaLaunchAttributeCooperative;
        attr.val.cooperative = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = B.cooperative ? 1 : 0;
        // chunk partials: at most 4 Gp + n_meshes chunks (two values each)
        TAD_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_b_pcg_persistent<d, T>, B.n_meshes, (const int64_t*)B.row_off, pth,
                                        (const int32_t*)P.bptr, (const int32_t*)P.bcol, (const T*)H, xs, r, z, p, Ap,
                                        (const T*)dinv, B.partials, 4 * Gp + B.n_meshes, B.counters, B.S, B.pcg_iters, gb,
                                        B.bar + 48));
    }
    k_b_to_double<T><<<G, TH, 0, s>>>(n, xs, P.dx);
    // 3. line search: d.g per mesh (with the g at x, before the full step's
    // assembly replaces it).  The full step s = 1 is evaluated by the full
    // element kernels and assembly at x + d, which are the next iteration's
    // derivatives for every mesh that takes it (as in the single-problem
    // loop); its energies are trial 0.  Then batches of 8 and 7 energy-only
    // trials at x + s d run only while some mesh has not accepted a step (the
    // trial kernels read the count the selection leaves and return at once
    // when it is 0); per-mesh choice and step.
    k_b_dot<d><<<G, TH, 0, s>>>(B.vch, B.n_vch, B.vmcb, B.vmce, P.dx, P.g, B.partials, B.counters, B.S.dg);
    k_b_add<d><<<G, TH, 0, s>>>(n, B.x, P.dx, B.xt);
    st = eval_elements(P, TAD_MODE_HESSIAN_PROJ, B.xt, eps, prec);
    if (st != TAD_OK) return st;
    k_b_reduce_rows<<<dim3(G, 1), TH, 0, s>>>(B.ech, B.n_ech, B.emcb, B.emce, P.ef, P.n_elem_total, B.partials,
                                              B.counters, B.S.ftr, LS_TRIALS);
    launch_assemble_grad_newton(P, prec, prec == TAD_PREC_MIXED);
    launch_assemble_hess(P, prec);
    for (int t0 = 0; t0 < LS_TRIALS;)
    {
        const int nb = t0 == 0 ? 1 : std::min(LS_BATCH, LS_TRIALS - t0);
        if (t0 > 0)
        {
            double* save = P.steps;
            P.steps = B.steps + t0;
            P.launch_guard = B.S.searching;
            st = eval_elements(P, TAD_MODE_LINESEARCH, B.x, 0.0, P.precision, P.dx, nb);
            P.steps = save;
            P.launch_guard = nullptr;
            if (st != TAD_OK) return st;
            k_b_reduce_rows<<<dim3(G, nb), TH, 0, s>>>(B.ech, B.n_ech, B.emcb, B.emce, P.ef, P.n_elem_total,
                                                       B.partials, B.counters, B.S.ftr + t0, LS_TRIALS, B.S.searching);
        }
        TAD_CUDA_TRY(cudaMemsetAsync(B.S.searching, 0, sizeof(int32_t), s));
        k_b_ls_select<<<(B.n_meshes + 255) / 256, 256, 0, s>>>(B.n_meshes, t0, nb, B.steps, P.settings.ls_armijo, B.S);
        // the meshes that rejected the full step need an evaluation at their new x
        if (t0 == 0)
            TAD_CUDA_TRY(cudaMemcpyAsync(B.S.need_eval, B.S.searching, sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
        t0 += nb;
    }
    k_b_axpy<d><<<G, TH, 0, s>>>(B.vch, B.n_vch, B.x, P.dx, B.S, 0);
    k_b_adopt_f<<<(B.n_meshes + 255) / 256, 256, 0, s>>>(B.n_meshes, B.S);
    TAD_CUDA_TRY(cudaGetLastError());
    return TAD_OK;
}

template <int d>
static tad_status capture(Batch& B, int prec, double eps)
{
    Problem& P = *B.P;
    if (B.graph) { cudaGraphExecDestroy(B.graph); B.graph = nullptr; }
    cudaGraph_t g;
    TAD_CUDA_TRY(cudaStreamBeginCapture(P.stream, cudaStreamCaptureModeThreadLocal));
    tad_status st = prec == TAD_PREC_MIXED ? record_iteration<d, float>(B, prec, eps) : record_iteration<d, double>(B, prec, eps);
    cudaGraph_t tmp;
    cudaError_t e = cudaStreamEndCapture(P.stream, &tmp);
    if (st != TAD_OK) { if (e == cudaSuccess) cudaGraphDestroy(tmp); return st; }
    TAD_CUDA_TRY(e);
    g = tmp;
    TAD_CUDA_TRY(cudaGraphInstantiate(&B.graph, g, 0));
    cudaGraphDestroy(g);
    return TAD_OK;
}

static tad_status batch_capture(Batch& B, double eps)
{
    switch (B.P->d)
    {
    case 1: return capture<1>(B, B.P->precision, eps);
    case 2: return capture<2>(B, B.P->precision, eps);
    default: return capture<3>(B, B.P->precision, eps);
    }
}

} // namespace tadlib

using namespace tadlib;

struct tad_batch : public tadlib::Batch {};

extern "C" {

TAD_API tad_status tad_batch_create(int var_dim, int n_meshes, const int64_t* n_handles, const tad_settings* settings,
                                    tad_batch** out)
{
    if (!out || !n_handles || n_meshes < 1 || n_meshes > 4096) return batch_fail(TAD_ERR_ARG, "bad batch arguments (1..4096 meshes)");
    *out = nullptr;
    tad_batch* B = new tad_batch();
    B->n_meshes = n_meshes;
    B->vert_off.assign(n_meshes + 1, 0);
    for (int m = 0; m < n_meshes; ++m)
    {
        if (n_handles[m] <= 0) { delete B; return batch_fail(TAD_ERR_ARG, "every mesh needs at least one handle"); }
        B->vert_off[m + 1] = B->vert_off[m] + n_handles[m];
    }
    // each mesh solves with block Jacobi (the batched PCG has no V-cycle), so the
    // concatenated problem builds no AMG hierarchy
    tad_settings st;
    if (settings) st = *settings;
    else tad_settings_default(&st);
    st.preconditioner = 0;
    tad_status s = tad_problem_create(var_dim, B->vert_off[n_meshes], &st, &B->P);
    if (s != TAD_OK) { delete B; return s; }
    *out = B;
    return TAD_OK;
}

TAD_API tad_status tad_batch_add_elements(tad_batch* B, int energy, int valence, const int64_t* n_elem_per_mesh,
                                          const int32_t* handles_h, const double* params_h, int n_params)
{
    if (!B || !n_elem_per_mesh) return batch_fail(TAD_ERR_ARG, "NULL argument");
    int64_t total = 0;
    for (int m = 0; m < B->n_meshes; ++m) total += n_elem_per_mesh[m];
    std::vector<int32_t> h(handles_h, handles_h + total * valence);
    int64_t e = 0;
    for (int m = 0; m < B->n_meshes; ++m)
        for (int64_t k = 0; k < n_elem_per_mesh[m]; ++k, ++e)
            for (int a = 0; a < valence; ++a)
            {
                int32_t& v = h[e * valence + a];
                if (v < 0 || v >= B->vert_off[m + 1] - B->vert_off[m]) return batch_fail(TAD_ERR_ARG, "mesh-local handle out of range");
                v += (int32_t)B->vert_off[m];
            }
    tad_status s = tad_add_elements(B->P, energy, valence, total, h.data(), params_h, n_params);
    if (s != TAD_OK) return s;
    B->elem_cnt.emplace_back(n_elem_per_mesh, n_elem_per_mesh + B->n_meshes);
    return TAD_OK;
}

__global__ void k_b_noop() {}

/* whether a cooperative launch can be recorded in a stream capture here (a
   one-block no-op, captured on a private stream and instantiated) */
static bool cooperative_capture_works()
{
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) { cudaGetLastError(); return false; }
    bool ok = false;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess)
    {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(1);
        cfg.blockDim = dim3(32);
        cfg.stream = st;
        cudaLaunchAttribute attr;
        attr.id = cudaLaunchAttributeCooperative;
        attr.val.cooperative = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        const cudaError_t e1 = cudaLaunchKernelEx(&cfg, k_b_noop);
        cudaGraph_t g = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(st, &g);
        if (e1 == cudaSuccess && e2 == cudaSuccess && g)
        {
            cudaGraphExec_t ge = nullptr;
            ok = cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
            if (ge) cudaGraphExecDestroy(ge);
        }
        if (g) cudaGraphDestroy(g);
    }
    cudaGetLastError();
    cudaStreamDestroy(st);
    return ok;
}

static tad_status batch_prepare(tad_batch* B)
{
    tad_status s = ensure_finalized(*B->P);
    if (s != TAD_OK) return s;
    if (!B->counters)
    {
        int sms = 0;
        TAD_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, B->P->device));
        B->sms = std::max(sms, 1);
        B->grid = 4 * B->sms;
        B->cooperative = cooperative_capture_works();
        TAD_CUDA_TRY(cudaMalloc(&B->bar, 64 * sizeof(unsigned)));
        TAD_CUDA_TRY(cudaMemset(B->bar, 0, 64 * sizeof(unsigned)));
        TAD_CUDA_TRY(cudaMalloc(&B->counters, (size_t)LS_TRIALS * 4096 * sizeof(unsigned)));
        TAD_CUDA_TRY(cudaMemset(B->counters, 0, (size_t)LS_TRIALS * 4096 * sizeof(unsigned)));
        const int nm = B->n_meshes;
        TAD_CUDA_TRY(cudaMalloc(&B->scal, (size_t)nm * (LS_TRIALS + 13) * sizeof(double)));
        TAD_CUDA_TRY(cudaMemset(B->scal, 0, (size_t)nm * (LS_TRIALS + 13) * sizeof(double)));
        TAD_CUDA_TRY(cudaMalloc(&B->iscal, (size_t)(nm * 5 + 3) * sizeof(int32_t)));
        TAD_CUDA_TRY(cudaMemset(B->iscal, 0, (size_t)(nm * 5 + 3) * sizeof(int32_t)));
        double* q = B->scal;
        B->S.f = q; q += nm;
        B->S.ftr = q; q += (size_t)nm * LS_TRIALS;
        B->S.gg = q; q += nm;
        B->S.dg = q; q += nm;
        B->S.rz = q; q += nm;
        B->S.bb = q; q += nm;
        B->S.tol2 = q; q += nm;
        B->S.alpha = q; q += nm;
        B->S.beta = q; q += nm;
        B->S.rr = q; q += nm;
        B->S.step = q; q += nm;
        B->S.f_start = q; q += nm;
        B->S.pap = q; q += nm;
        B->S.done = B->iscal;
        B->S.iters = B->iscal + nm;
        B->S.choice = B->iscal + 2 * nm;
        B->S.searching = B->iscal + 3 * nm;
        B->S.stalled = B->iscal + 4 * nm + 2;
        B->S.need_eval = B->iscal + 5 * nm + 2;
        TAD_CUDA_TRY(cudaMalloc(&B->steps, LS_TRIALS * sizeof(double)));
        std::vector<double> st(LS_TRIALS);
        double sv = 1.0;
        for (int j = 0; j < LS_TRIALS; ++j) { st[j] = sv; sv *= B->P->settings.ls_shrink; }
        TAD_CUDA_TRY(cudaMemcpy(B->steps, st.data(), LS_TRIALS * sizeof(double), cudaMemcpyHostToDevice));
        TAD_CUDA_TRY(cudaMallocHost(&B->fh, (size_t)nm * sizeof(double)));
        TAD_CUDA_TRY(cudaMalloc(&B->x, B->P->n_vars * sizeof(double)));
        TAD_CUDA_TRY(cudaMalloc(&B->xt, B->P->n_vars * sizeof(double)));
        s = batch_setup_chunks(*B);
        if (s != TAD_OK) return s;
    }
    return TAD_OK;
}

/* n_iters batched Newton iterations on device x (x_d, concatenated meshes).
   f_hist_h (optional): [n_iters + 1][n_meshes] energies. */
TAD_API tad_status tad_batch_newton_solve_d(tad_batch* B, double* x_d, int n_iters, double eps, double* f_hist_h)
{
    if (!B || !x_d) return batch_fail(TAD_ERR_ARG, "NULL argument");
    TAD_CUDA_TRY(cudaSetDevice(B->P->device));
    tad_status s = batch_prepare(B);
    if (s != TAD_OK) return s;
    Problem& P = *B->P;
    const int nm = B->n_meshes;
    B->pcg_iters = std::max(1, std::min(P.settings.pcg_max_iters, 4096));
    B->pcg_tol = P.settings.pcg_rel_tol;
    TAD_CUDA_TRY(cudaMemcpyAsync(B->x, x_d, P.n_vars * 8, cudaMemcpyDeviceToDevice, P.stream));
    // a new start: no mesh stalled, and the first iteration evaluates at x
    TAD_CUDA_TRY(cudaMemsetAsync(B->S.stalled, 0, (size_t)nm * sizeof(int32_t), P.stream));
    TAD_CUDA_TRY(cudaMemsetAsync(B->S.need_eval, 1, sizeof(int32_t), P.stream));
    if (!B->graph)
    {
        s = batch_capture(*B, eps);
        if (s != TAD_OK) return s;
    }
    for (int it = 0; it < n_iters; ++it)
    {
        TAD_CUDA_TRY(cudaGraphLaunch(B->graph, P.stream));
        P.n_launches += 1;
        if (f_hist_h)
        {
            TAD_CUDA_TRY(cudaMemcpyAsync(B->fh, B->S.f_start, nm * 8, cudaMemcpyDeviceToHost, P.stream));
            TAD_CUDA_TRY(cudaStreamSynchronize(P.stream));
            std::copy(B->fh, B->fh + nm, f_hist_h + (size_t)it * nm);
        }
    }
    if (f_hist_h)
    {
        // energy at the final x
        s = eval_elements(P, TAD_MODE_VALUE, B->x, 0.0, TAD_PREC_FP64);
        if (s != TAD_OK) return s;
        k_b_reduce_rows<<<dim3(B->grid, 1), B->threads, 0, P.stream>>>(B->ech, B->n_ech, B->emcb, B->emce, P.ef,
                                                                      P.n_elem_total, B->partials, B->counters, B->S.f, 1);
        TAD_CUDA_TRY(cudaMemcpyAsync(B->fh, B->S.f, nm * 8, cudaMemcpyDeviceToHost, P.stream));
        TAD_CUDA_TRY(cudaStreamSynchronize(P.stream));
        std::copy(B->fh, B->fh + nm, f_hist_h + (size_t)n_iters * nm);
    }
    TAD_CUDA_TRY(cudaMemcpyAsync(x_d, B->x, P.n_vars * 8, cudaMemcpyDeviceToDevice, P.stream));
    TAD_CUDA_TRY(cudaStreamSynchronize(P.stream));
    return check_device_error(P);
}

TAD_API tad_status tad_batch_newton_solve(tad_batch* B, double* x_h, int n_iters, double eps, double* f_hist_h)
{
    if (!B || !x_h) return batch_fail(TAD_ERR_ARG, "NULL argument");
    TAD_CUDA_TRY(cudaSetDevice(B->P->device));
    tad_status s = batch_prepare(B);
    if (s != TAD_OK) return s;
    Problem& P = *B->P;
    TAD_CUDA_TRY(cudaMemcpyAsync(P.x, x_h, P.n_vars * 8, cudaMemcpyHostToDevice, P.stream));
    s = tad_batch_newton_solve_d(B, P.x, n_iters, eps, f_hist_h);
    if (s != TAD_OK) return s;
    TAD_CUDA_TRY(cudaMemcpyAsync(x_h, P.x, P.n_vars * 8, cudaMemcpyDeviceToHost, P.stream));
    TAD_CUDA_TRY(cudaStreamSynchronize(P.stream));
    return TAD_OK;
}

/* Autotuner: times one captured batched Newton iteration for each candidate
   (block rows per chunk x threads per block) on the batch's current x and
   keeps the fastest.  Candidates are measured over three iterations after
   one warm replay, with CUDA events on the batch's stream; the state x is
   restored afterwards.
   best3 (optional): [chunk_rows, threads, ms]. */
TAD_API tad_status tad_batch_autotune(tad_batch* B, const double* x_d, double eps, double* best3)
{
    if (!B || !x_d) return batch_fail(TAD_ERR_ARG, "NULL argument");
    TAD_CUDA_TRY(cudaSetDevice(B->P->device));
    tad_status s = batch_prepare(B);
    if (s != TAD_OK) return s;
    Problem& P = *B->P;
    B->pcg_iters = std::max(1, std::min(P.settings.pcg_max_iters, 4096));
    B->pcg_tol = P.settings.pcg_rel_tol;
    // each candidate is timed over TUNE_ITERS consecutive iterations from x:
    // the linear solves get harder as the meshes converge, and the first
    // iteration alone favours the launch shape of the easy solves
    constexpr int TUNE_ITERS = 3;
    // element / vector chunk rows x threads per block x blocks per SM of the
    // persistent PCG (the PCG's chunks follow the meshes still iterating)
    const int rows_c[] = {512, 2048};
    const int thr_c[] = {128, 256};
    const int pb_c[] = {4, 8, 16};
    double best = 1e30;
    int br = B->chunk_rows, bt = B->threads, bp = B->pb_per_sm;
    for (int rows : rows_c)
        for (int thr : thr_c)
            for (int pb : pb_c)
        {
            B->chunk_rows = rows;
            B->threads = thr;
            B->pb_per_sm = pb;
            s = batch_setup_chunks(*B);
            if (s != TAD_OK) return s;
            s = batch_capture(*B, eps);
            if (s != TAD_OK) return s;
            float ms = 0.f;
            TAD_CUDA_TRY(cudaMemcpyAsync(B->x, x_d, P.n_vars * 8, cudaMemcpyDeviceToDevice, P.stream));
            TAD_CUDA_TRY(cudaMemsetAsync(B->S.stalled, 0, (size_t)B->n_meshes * sizeof(int32_t), P.stream));
            TAD_CUDA_TRY(cudaMemsetAsync(B->S.need_eval, 1, sizeof(int32_t), P.stream));
            TAD_CUDA_TRY(cudaGraphLaunch(B->graph, P.stream));
            TAD_CUDA_TRY(cudaMemcpyAsync(B->x, x_d, P.n_vars * 8, cudaMemcpyDeviceToDevice, P.stream));
            TAD_CUDA_TRY(cudaMemsetAsync(B->S.stalled, 0, (size_t)B->n_meshes * sizeof(int32_t), P.stream));
            TAD_CUDA_TRY(cudaMemsetAsync(B->S.need_eval, 1, sizeof(int32_t), P.stream));
            cudaEventRecord(P.ev[5], P.stream);
            for (int k = 0; k < TUNE_ITERS; ++k) TAD_CUDA_TRY(cudaGraphLaunch(B->graph, P.stream));
            cudaEventRecord(P.ev[6], P.stream);
            TAD_CUDA_TRY(cudaEventSynchronize(P.ev[6]));
            cudaEventElapsedTime(&ms, P.ev[5], P.ev[6]);
            ms /= TUNE_ITERS;
            if (ms < best) { best = ms; br = rows; bt = thr; bp = pb; }
        }
    B->chunk_rows = br;
    B->threads = bt;
    B->pb_per_sm = bp;
    s = batch_setup_chunks(*B);
    if (s != TAD_OK) return s;
    s = batch_capture(*B, eps);
    if (s != TAD_OK) return s;
    TAD_CUDA_TRY(cudaMemcpyAsync(B->x, x_d, P.n_vars * 8, cudaMemcpyDeviceToDevice, P.stream));
    TAD_CUDA_TRY(cudaStreamSynchronize(P.stream));
    if (best3) { best3[0] = br; best3[1] = bt; best3[2] = best; }
    return TAD_OK;
}

TAD_API tad_status tad_batch_set_chunking(tad_batch* B, int chunk_rows, int threads)
{
    if (!B) return batch_fail(TAD_ERR_ARG, "NULL argument");
    if (chunk_rows < 32 || chunk_rows > (1 << 20) || threads < 32 || threads > 1024 || threads % 32 != 0)
        return batch_fail(TAD_ERR_ARG, "chunk_rows in [32, 2^20], threads a multiple of 32 in [32, 1024]");
    TAD_CUDA_TRY(cudaSetDevice(B->P->device));
    B->chunk_rows = chunk_rows;
    B->threads = threads;
    if (B->graph) { TAD_CUDA_TRY(cudaStreamSynchronize(B->P->stream)); cudaGraphExecDestroy(B->graph); B->graph = nullptr; }
    if (B->counters) return batch_setup_chunks(*B);   // prepared: rebuild the chunk lists now
    return TAD_OK;
}

TAD_API tad_status tad_batch_problem(tad_batch* B, tad_problem** p)
{
    if (!B || !p) return batch_fail(TAD_ERR_ARG, "NULL argument");
    *p = B->P;
    return TAD_OK;
}

TAD_API tad_status tad_batch_destroy(tad_batch* B)
{
    if (!B) return TAD_OK;
    if (B->P) cudaStreamSynchronize(B->P->stream);
    if (B->graph) cudaGraphExecDestroy(B->graph);
    void* bufs[] = {B->vch, B->ech, B->vmcb, B->vmce, B->emcb, B->emce, B->partials, B->counters, B->scal, B->iscal,
                    B->steps, B->x, B->xt, B->row_off, B->bar};
    for (void* b : bufs) if (b) cudaFree(b);
    if (B->fh) cudaFreeHost(B->fh);
    tad_problem_destroy(B->P);
    delete B;
    return TAD_OK;
}

} // extern "C"
