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
 * so every per-mesh reduction is deterministic.  The PCG kernels use a chunk
 * list rebuilt on the device from the meshes still iterating (at PCG
 * iterations 0-4, 6, 8, 12, 16, ...), cut so that the remaining rows spread
 * over the whole grid, one block per chunk.
 *
 * One Newton iteration (elements -> f -> assembly, only when some mesh did
 * not take the previous full step -> PCG with a fixed number of iterations,
 * each mesh stopping at its own tolerance -> the full step, evaluated by the
 * element kernels and assembly at x + d, which are the next iteration's
 * derivatives -> batches of 8 and 7 energy-only trials while some mesh has
 * not accepted one -> per-mesh step) has a fixed launch sequence and is
 * captured once as a CUDA graph; the host replays one graph per iteration.
 * Kernels of the PCG iterations after every mesh has converged, and of the
 * trials after every mesh has accepted a step, return at once (device
 * counters).
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
    int32_t* pcg_active;  // [2] meshes still iterating after the last two PCG updates (ping-pong)
    int32_t* stalled;     // [m] no trial step passed the Armijo test: x stays, and so would every later
                          // iteration's result; the mesh is left out of the PCG and the line search
                          // until the next solve call
    int32_t* need_eval;   // meshes that rejected the full step in the last iteration (0: the
                          // derivatives assembled at x + d are those of every mesh's new x)
    double* f_start;      // [m] energy at the start of the last iteration (the history)
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

/* The PCG kernels' chunk list, rebuilt on the device from the meshes still
   iterating: their rows are cut into chunks of C = max(min_rows,
   ceil(R / (2 G))) rows for R active rows and a grid of G blocks, so the
   remaining work spreads over the whole grid however few meshes are left
   (the last meshes to converge are the largest ones, whose rows would
   otherwise sit in a few long chunks, one block each).  At most 2 G +
   n_meshes chunks.  One block; thread t owns a contiguous run of meshes,
   and the chunk offsets are an exclusive scan of the per-thread counts.
   active: skip the rebuild when no mesh is iterating (0). */
constexpr int CHUNK_BUILD_THREADS = 1024;

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

__global__ void __launch_bounds__(CHUNK_BUILD_THREADS) k_b_pcg_chunks(int n_meshes, const int64_t* __restrict__ row_off,
                                                                      const int32_t* __restrict__ done, int grid,
                                                                      int min_rows, const int32_t* active, Chunk* ch,
                                                                      int32_t* mcb, int32_t* mce, int32_t* n_ch)
{
    if (active && *active == 0) return;
    __shared__ long long tot_ll[32];
    __shared__ int tot_i[32];
    const int per = (n_meshes + CHUNK_BUILD_THREADS - 1) / CHUNK_BUILD_THREADS;
    const int m0 = min(n_meshes, (int)threadIdx.x * per), m1 = min(n_meshes, m0 + per);
    long long rows = 0;
    for (int m = m0; m < m1; ++m)
        if (!done[m]) rows += row_off[m + 1] - row_off[m];
    long long R;
    (void)block_exclusive_scan<long long>(rows, tot_ll, R);
    const long long C = max((long long)min_rows, (R + 2LL * grid - 1) / (2LL * grid));
    int cnt = 0;
    for (int m = m0; m < m1; ++m)
        if (!done[m]) cnt += (int)((row_off[m + 1] - row_off[m] + C - 1) / C);
    int total;
    int off = block_exclusive_scan<int>(cnt, tot_i, total);
    for (int m = m0; m < m1; ++m)
    {
        mcb[m] = off;
        if (!done[m])
            for (long long b = row_off[m]; b < row_off[m + 1]; b += C)
                ch[off++] = Chunk{m, (int32_t)b, (int32_t)min((long long)row_off[m + 1], b + C)};
        mce[m] = off;
    }
    if (threadIdx.x == 0) *n_ch = total;
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

/* per mesh still iterating: Ap = H z + beta Ap, p = z + beta p (H p_new =
   H z + beta H p_old, as in the single-problem PCG), alpha = rz / p.Ap.
   active: meshes still iterating after the previous update (0: every block
   returns at once -- the rest of the iteration budget is idle) */
template <int d, typename T>
__global__ void k_b_spmv(const Chunk* ch, const int32_t* n_ch, int stride, const int32_t* mcb, const int32_t* mce,
                         const int32_t* bptr, const int32_t* bcol, const T* H, const T* z, T* p, T* Ap, double* partials,
                         unsigned* counters, BatchScalars S, const int32_t* active)
{
    if (*active == 0) return;
    const int n_chunks = *n_ch;
    for (int ci = blockIdx.x; ci < n_chunks; ci += gridDim.x)
    {
        const Chunk c = ch[ci];
        if (S.done[c.mesh]) continue;
        const T beta = from_double<T>(S.beta[c.mesh]);
        T part = T(0);
        for (int64_t u = c.begin + threadIdx.x; u < c.end; u += blockDim.x)
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
        double v[1] = {as_double(part)}, tot[1];
        if (seg_finish<1>(ci, c.mesh, v, partials, stride, counters, mcb, mce, tot) && threadIdx.x == 0)
        {
            const int m = c.mesh;
            if (!(tot[0] > 0.0) || !isfinite(tot[0])) { S.done[m] = 1; S.alpha[m] = 0.0; }
            else S.alpha[m] = S.rz[m] / tot[0];
        }
    }
}

/* x += alpha p, r -= alpha Ap, z = D^-1 r; rz, rr and beta per mesh.  A mesh
   that converged, reached max_iters or went non-finite is done; the others
   are counted into active_out (zeroed before), which the next SpMV and
   update read as their active_in */
template <int d, typename T>
__global__ void k_b_update(const Chunk* ch, const int32_t* n_ch, int stride, const int32_t* mcb, const int32_t* mce,
                           T* x, T* r, T* z, const T* p, const T* Ap, const T* dinv, double* partials, unsigned* counters,
                           BatchScalars S, int max_iters, const int32_t* active_in, int32_t* active_out)
{
    if (*active_in == 0) return;
    const int n_chunks = *n_ch;
    for (int ci = blockIdx.x; ci < n_chunks; ci += gridDim.x)
    {
        const Chunk c = ch[ci];
        if (S.done[c.mesh]) continue;
        const T alpha = from_double<T>(S.alpha[c.mesh]);
        T acc_rz = T(0), acc_rr = T(0);
        for (int64_t u = c.begin + threadIdx.x; u < c.end; u += blockDim.x)
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
        if (seg_finish<2>(ci, c.mesh, v, partials, stride, counters, mcb, mce, tot) && threadIdx.x == 0)
        {
            const int m = c.mesh;
            S.beta[m] = tot[0] / S.rz[m];
            S.rz[m] = tot[0];
            S.rr[m] = tot[1];
            S.iters[m] += 1;
            if (tot[1] <= S.tol2[m] || S.iters[m] >= max_iters || !isfinite(tot[1])) S.done[m] = 1;
            else atomicAdd(active_out, 1);
        }
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
    // PCG chunk list built on the device (k_b_pcg_chunks): capacity, list,
    // per-mesh ranges, count; per-mesh row offsets
    int pch_cap = 0;
    Chunk* pch = nullptr;
    int32_t *pmcb = nullptr, *pmce = nullptr, *n_pch = nullptr;
    int64_t* row_off = nullptr;
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
    B.pch_cap = 2 * B.grid + B.n_meshes;
    if (B.pch) { cudaFree(B.pch); B.pch = nullptr; }
    TAD_CUDA_TRY(cudaMalloc(&B.pch, (size_t)B.pch_cap * sizeof(Chunk)));
    if (!B.pmcb)
    {
        TAD_CUDA_TRY(cudaMalloc(&B.pmcb, (size_t)B.n_meshes * sizeof(int32_t)));
        TAD_CUDA_TRY(cudaMalloc(&B.pmce, (size_t)B.n_meshes * sizeof(int32_t)));
        TAD_CUDA_TRY(cudaMalloc(&B.n_pch, sizeof(int32_t)));
        TAD_CUDA_TRY(upload(&B.row_off, B.vert_off));
    }
    if (B.partials) cudaFree(B.partials);
    const size_t n_part = std::max<size_t>((size_t)std::max(B.n_vch, B.n_ech) * LS_TRIALS, (size_t)B.pch_cap) * 2;
    TAD_CUDA_TRY(cudaMalloc(&B.partials, n_part * sizeof(double)));
    return TAD_OK;
}

/* PCG iterations before which the chunk list is rebuilt (0, 1, 2, 3, 4, 6,
   8, 12, 16, 24, 32, 48, ...): between rebuilds the list is a superset of
   the meshes still iterating, whose finished chunks are skipped */
static bool rebuild_chunks_before(int it)
{
    if (it <= 4) return true;
    const int q = it % 3 == 0 ? it / 3 : it;
    return (q & (q - 1)) == 0;
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
    // 2. PCG, per-mesh tolerance.  Iteration it reads the active count the
    // previous update left in pcg_active[it & 1] and counts into the other
    // slot; the first count is set nonzero so the first iteration runs.
    k_b_pcg_init<d, T><<<G, TH, 0, s>>>(B.vch, B.n_vch, B.vmcb, B.vmce, P.rhs, P.diag, H, xs, r, z, p, Ap, dinv,
                                        B.partials, B.counters, B.S, B.pcg_tol);
    TAD_CUDA_TRY(cudaMemsetAsync(B.S.pcg_active, 1, sizeof(int32_t), s));
    for (int it = 0; it < B.pcg_iters; ++it)
    {
        const int32_t* in = B.S.pcg_active + (it & 1);
        int32_t* out = B.S.pcg_active + ((it + 1) & 1);
        if (rebuild_chunks_before(it))
            k_b_pcg_chunks<<<1, CHUNK_BUILD_THREADS, 0, s>>>(B.n_meshes, B.row_off, B.S.done, G, TH, in, B.pch, B.pmcb,
                                                             B.pmce, B.n_pch);
        // one block per chunk slot (blocks past the list's length return at
        // once): the block scheduler balances chunks of uneven length
        k_b_spmv<d, T><<<B.pch_cap, TH, 0, s>>>(B.pch, B.n_pch, B.pch_cap, B.pmcb, B.pmce, P.bptr, P.bcol, H, z, p,
                                                Ap, B.partials, B.counters, B.S, in);
        TAD_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(int32_t), s));
        k_b_update<d, T><<<B.pch_cap, TH, 0, s>>>(B.pch, B.n_pch, B.pch_cap, B.pmcb, B.pmce, xs, r, z, p, Ap, dinv,
                                                  B.partials, B.counters, B.S, B.pcg_iters, in, out);
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
    tad_status s = tad_problem_create(var_dim, B->vert_off[n_meshes], settings, &B->P);
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

static tad_status batch_prepare(tad_batch* B)
{
    tad_status s = ensure_finalized(*B->P);
    if (s != TAD_OK) return s;
    if (!B->counters)
    {
        int sms = 0;
        TAD_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, B->P->device));
        B->grid = 4 * std::max(sms, 1);
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
        B->S.done = B->iscal;
        B->S.iters = B->iscal + nm;
        B->S.choice = B->iscal + 2 * nm;
        B->S.searching = B->iscal + 3 * nm;
        B->S.pcg_active = B->iscal + 4 * nm;
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
    const int rows_c[] = {256, 512, 1024, 2048, 4096};
    const int thr_c[] = {128, 256};
    double best = 1e30;
    int br = B->chunk_rows, bt = B->threads;
    for (int rows : rows_c)
        for (int thr : thr_c)
        {
            B->chunk_rows = rows;
            B->threads = thr;
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
            if (ms < best) { best = ms; br = rows; bt = thr; }
        }
    B->chunk_rows = br;
    B->threads = bt;
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
                    B->steps, B->x, B->xt, B->pch, B->pmcb, B->pmce, B->n_pch, B->row_off};
    for (void* b : bufs) if (b) cudaFree(b);
    if (B->fh) cudaFreeHost(B->fh);
    tad_problem_destroy(B->P);
    delete B;
    return TAD_OK;
}

} // extern "C"
