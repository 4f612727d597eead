/*
 * Aggregation AMG preconditioner for the device PCG.
 *
 * Block-Jacobi PCG needs O(sqrt(cond)) iterations, thousands on the large
 * meshes once Newton's tolerance tightens.  A solve that has not converged
 * after its first block-Jacobi iterations restarts with conjugate gradients
 * preconditioned by one V-cycle of this hierarchy (solver.cu, pcg_core).
 *
 * Hierarchy (built once per sparsity pattern, on the host, when first
 * needed): greedy aggregation of the block graph -- a vertex whose
 * neighbours are all free roots an aggregate of its one-ring; vertices left
 * over join the aggregate of their first aggregated neighbour, isolated ones
 * form their own -- repeated until at most AMG_COARSE_ROWS block rows remain.
 * The prolongation is piecewise constant per aggregate, so each coarse block
 * A_c(I, J) = sum of the fine blocks A(u, v) with u in I, v in J (Galerkin
 * product P^T A P), formed on the device as an ordered gather-sum over
 * precomputed fine-block lists (deterministic, no atomics), like the
 * assembly.  The d x d block structure is kept on every level.
 *
 * V-cycle (symmetric and positive definite, so CG stays valid): on each
 * level, one damped block-Jacobi step from zero, residual, restriction (sum
 * over the aggregate), coarse correction, prolongation, one damped
 * block-Jacobi step; on the coarsest level (<= AMG_COARSE_ROWS block rows)
 * AMG_COARSE_SWEEPS damped block-Jacobi steps from zero in a single thread
 * block.  The damping of each level is omega = AMG_OMEGA_FACTOR / rho, rho
 * the spectral radius of D^-1 A estimated by AMG_POWER_STEPS power
 * iterations on the device (kept in device memory, so the captured graph
 * needs no update): a fixed omega = 2/3 makes the smoother diverge on these
 * non-M-matrices (rho > 3) and the V-cycle indefinite.  All kernels return at
 * once when the PCG's stop flag is set, so chunks of iterations are captured
 * in a CUDA graph like the block-Jacobi PCG.  Vectors and values are kept in
 * the PCG's precision.
 */
#include <algorithm>
#include <vector>

#include "internal.hh"
#include "grid_reduce.cuh"
#include "bsr_kernels.cuh"

namespace tadlib {

constexpr int64_t AMG_COARSE_ROWS = 512;
constexpr int AMG_MAX_LEVELS = 12;
constexpr int AMG_COARSE_SWEEPS = 16;
constexpr int AMG_COARSE_THREADS = 512;
constexpr int AMG_POWER_STEPS = 12;
constexpr double AMG_OMEGA_FACTOR = 1.2;     // omega rho <= 2 while the estimate is >= 0.6 rho

/* ---- host: aggregation and coarse patterns -------------------------------- */
namespace {

struct HostLevel
{
    int64_t n = 0;
    std::vector<int32_t> bptr, bcol, diag;   // this level's BSR pattern
    std::vector<int32_t> agg;                // rows of the level above -> rows here
    std::vector<int32_t> aptr, aidx;         // rows here -> rows of the level above
    std::vector<int32_t> cptr, cidx;         // blocks here -> blocks of the level above
};

std::vector<int32_t> aggregate(int64_t n, const std::vector<int32_t>& bptr, const std::vector<int32_t>& bcol, int64_t& nc)
{
    std::vector<int32_t> agg(n, -1);
    nc = 0;
    for (int64_t u = 0; u < n; ++u)
    {
        if (agg[u] >= 0) continue;
        bool free_ring = true;
        for (int32_t q = bptr[u]; q < bptr[u + 1] && free_ring; ++q) free_ring = agg[bcol[q]] < 0;
        if (!free_ring) continue;
        for (int32_t q = bptr[u]; q < bptr[u + 1]; ++q) agg[bcol[q]] = (int32_t)nc;
        agg[u] = (int32_t)nc++;
    }
    const std::vector<int32_t> first = agg;
    for (int64_t u = 0; u < n; ++u)
    {
        if (agg[u] >= 0) continue;
        for (int32_t q = bptr[u]; q < bptr[u + 1]; ++q)
            if (first[bcol[q]] >= 0) { agg[u] = first[bcol[q]]; break; }
    }
    for (int64_t u = 0; u < n; ++u)
        if (agg[u] < 0) agg[u] = (int32_t)nc++;
    return agg;
}

/* the coarse level under the fine pattern (fb, fc) for the aggregation agg */
void coarsen(int64_t nf, const std::vector<int32_t>& fb, const std::vector<int32_t>& fc, std::vector<int32_t> agg,
             int64_t nc, HostLevel& L)
{
    L.n = nc;
    L.agg = std::move(agg);
    L.aptr.assign(nc + 1, 0);
    for (int64_t u = 0; u < nf; ++u) ++L.aptr[L.agg[u] + 1];
    for (int64_t I = 0; I < nc; ++I) L.aptr[I + 1] += L.aptr[I];
    L.aidx.resize(nf);
    {
        std::vector<int32_t> fill(L.aptr.begin(), L.aptr.end() - 1);
        for (int64_t u = 0; u < nf; ++u) L.aidx[fill[L.agg[u]]++] = (int32_t)u;
    }
    // coarse columns per coarse row: the aggregates of the members' neighbours
    L.bptr.assign(nc + 1, 0);
    L.bcol.clear();
    std::vector<int32_t> cols;
    for (int64_t I = 0; I < nc; ++I)
    {
        cols.clear();
        for (int32_t a = L.aptr[I]; a < L.aptr[I + 1]; ++a)
        {
            const int32_t u = L.aidx[a];
            for (int32_t q = fb[u]; q < fb[u + 1]; ++q) cols.push_back(L.agg[fc[q]]);
        }
        std::sort(cols.begin(), cols.end());
        cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
        L.bcol.insert(L.bcol.end(), cols.begin(), cols.end());
        L.bptr[I + 1] = (int32_t)L.bcol.size();
    }
    L.diag.assign(nc, -1);
    for (int64_t I = 0; I < nc; ++I)
    {
        const auto it = std::lower_bound(L.bcol.begin() + L.bptr[I], L.bcol.begin() + L.bptr[I + 1], (int32_t)I);
        if (it != L.bcol.begin() + L.bptr[I + 1] && *it == I) L.diag[I] = (int32_t)(it - L.bcol.begin());
    }
    // fine block -> coarse block, then the lists per coarse block in fine block order
    const int64_t nbf = fb[nf], nbc = (int64_t)L.bcol.size();
    std::vector<int32_t> target(nbf);
    for (int64_t u = 0; u < nf; ++u)
    {
        const int32_t I = L.agg[u];
        for (int32_t q = fb[u]; q < fb[u + 1]; ++q)
        {
            const int32_t J = L.agg[fc[q]];
            const auto it = std::lower_bound(L.bcol.begin() + L.bptr[I], L.bcol.begin() + L.bptr[I + 1], J);
            target[q] = (int32_t)(it - L.bcol.begin());
        }
    }
    L.cptr.assign(nbc + 1, 0);
    for (int64_t q = 0; q < nbf; ++q) ++L.cptr[target[q] + 1];
    for (int64_t b = 0; b < nbc; ++b) L.cptr[b + 1] += L.cptr[b];
    L.cidx.resize(nbf);
    std::vector<int32_t> fill(L.cptr.begin(), L.cptr.end() - 1);
    for (int64_t q = 0; q < nbf; ++q) L.cidx[fill[target[q]]++] = (int32_t)q;
}

template <typename X>
cudaError_t upload(X** d, const std::vector<X>& h)
{
    cudaError_t e = cudaMalloc((void**)d, std::max<size_t>(h.size(), 1) * sizeof(X));
    if (e == cudaSuccess && !h.empty()) e = cudaMemcpy(*d, h.data(), h.size() * sizeof(X), cudaMemcpyHostToDevice);
    return e;
}

} // namespace

static tad_status amg_fail(const char* m) { set_error(m); return TAD_ERR_CUDA; }

void amg_free(Problem& P)
{
    for (size_t l = 0; l < P.amg.size(); ++l)
    {
        AmgLevel& L = P.amg[l];
        if (l > 0)
            for (void* q : {(void*)L.bptr, (void*)L.bcol, (void*)L.diag, L.A})
                if (q) cudaFree(q);
        for (void* q : {(void*)L.agg, (void*)L.aptr, (void*)L.aidx, (void*)L.cptr, (void*)L.cidx, L.dinv, L.r, L.z, L.w, L.t})
            if (q) cudaFree(q);
    }
    P.amg.clear();
    if (P.amg_omega) { cudaFree(P.amg_omega); P.amg_omega = nullptr; }
}

/* pattern-level hierarchy (once per problem) */
static tad_status amg_build(Problem& P)
{
    if (!P.amg.empty()) return TAD_OK;
    const int d = P.d;
    std::vector<HostLevel> H;
    {
        // level 0 pattern from the problem's BSR arrays
        HostLevel L0;
        L0.n = P.n_handles;
        L0.bptr.assign(P.bptr_h.begin(), P.bptr_h.end());
        L0.bcol.assign(P.bcol_h.begin(), P.bcol_h.end());
        H.push_back(std::move(L0));
    }
    while ((int)H.size() < AMG_MAX_LEVELS && H.back().n > AMG_COARSE_ROWS)
    {
        const HostLevel& F = H.back();
        int64_t nc = 0;
        std::vector<int32_t> agg = aggregate(F.n, F.bptr, F.bcol, nc);
        if (nc >= F.n * 9 / 10) break;   // coarsening stalled
        HostLevel C;
        coarsen(F.n, F.bptr, F.bcol, std::move(agg), nc, C);
        H.push_back(std::move(C));
    }
    P.amg.resize(H.size());
    if (!P.amg_omega && cudaMalloc(&P.amg_omega, (AMG_MAX_LEVELS + 2) * sizeof(double)) != cudaSuccess)
        return amg_fail("AMG: device allocation failed");
    const size_t vb = sizeof(double);   // vectors and values sized for FP64, used as T
    for (size_t l = 0; l < H.size(); ++l)
    {
        AmgLevel& L = P.amg[l];
        const HostLevel& h = H[l];
        L.n = h.n;
        if (l == 0)
        {
            L.nb = P.nb;
            L.bptr = P.bptr; L.bcol = P.bcol; L.diag = P.diag;
        }
        else
        {
            L.nb = (int64_t)h.bcol.size();
            if (upload(&L.bptr, h.bptr) != cudaSuccess || upload(&L.bcol, h.bcol) != cudaSuccess ||
                upload(&L.diag, h.diag) != cudaSuccess || upload(&L.agg, h.agg) != cudaSuccess ||
                upload(&L.aptr, h.aptr) != cudaSuccess || upload(&L.aidx, h.aidx) != cudaSuccess ||
                upload(&L.cptr, h.cptr) != cudaSuccess || upload(&L.cidx, h.cidx) != cudaSuccess)
            {
                amg_free(P);
                return amg_fail("AMG: device allocation failed");
            }
            if (cudaMalloc(&L.A, std::max<int64_t>(L.nb, 1) * d * d * vb) != cudaSuccess) { amg_free(P); return amg_fail("AMG: device allocation failed"); }
        }
        if (cudaMalloc(&L.dinv, std::max<int64_t>(L.n, 1) * d * d * vb) != cudaSuccess ||
            cudaMalloc(&L.r, std::max<int64_t>(L.n, 1) * d * vb) != cudaSuccess ||
            cudaMalloc(&L.z, std::max<int64_t>(L.n, 1) * d * vb) != cudaSuccess ||
            cudaMalloc(&L.w, std::max<int64_t>(L.n, 1) * d * vb) != cudaSuccess ||
            cudaMalloc(&L.t, std::max<int64_t>(L.n, 1) * d * vb) != cudaSuccess)
        {
            amg_free(P);
            return amg_fail("AMG: device allocation failed");
        }
    }
    return TAD_OK;
}

/* ---- device kernels ---------------------------------------------------------- */
template <int d, typename T>
__global__ void k_amg_galerkin(int64_t nb, const int32_t* __restrict__ cptr, const int32_t* __restrict__ cidx,
                               const T* __restrict__ Af, T* __restrict__ Ac)
{
    GRID_STRIDE(b, nb)
    {
        T acc[d * d];
#pragma unroll
        for (int i = 0; i < d * d; ++i) acc[i] = T(0);
        for (int32_t q = cptr[b]; q < cptr[b + 1]; ++q)
        {
            const T* blk = Af + (int64_t)cidx[q] * d * d;
#pragma unroll
            for (int i = 0; i < d * d; ++i) acc[i] += blk[i];
        }
#pragma unroll
        for (int i = 0; i < d * d; ++i) Ac[b * d * d + i] = acc[i];
    }
}

#define AMG_STOP if (ds && *(volatile const int32_t*)&ds->done) return

/* coarsest level: AMG_COARSE_SWEEPS damped block-Jacobi steps from zero in
   one thread block (the rows are few; a launch per sweep would dominate) */
template <int d, typename T>
__global__ void __launch_bounds__(AMG_COARSE_THREADS) k_amg_coarse(int64_t n, const int32_t* __restrict__ bptr,
                                                                   const int32_t* __restrict__ bcol, const T* __restrict__ A,
                                                                   const T* __restrict__ dinv, const T* __restrict__ r,
                                                                   T* __restrict__ z, T* __restrict__ w,
                                                                   const double* __restrict__ omega_p, const DevScalars* ds)
{
    AMG_STOP;
    const T omega = (T)*omega_p;
    for (int64_t u = threadIdx.x; u < n; u += blockDim.x)
    {
        T rv[d], zv[d];
#pragma unroll
        for (int i = 0; i < d; ++i) rv[i] = r[u * d + i];
        apply_dinv<d, T>(dinv, u, rv, zv);
#pragma unroll
        for (int i = 0; i < d; ++i) z[u * d + i] = omega * zv[i];
    }
    __syncthreads();
    T* a = z;
    T* b = w;
    for (int k = 0; k < AMG_COARSE_SWEEPS; ++k)
    {
        for (int64_t u = threadIdx.x; u < n; u += blockDim.x)
        {
            T y[d];
#pragma unroll
            for (int i = 0; i < d; ++i) y[i] = r[u * d + i];
            for (int32_t q = bptr[u]; q < bptr[u + 1]; ++q)
            {
                const int64_t c = bcol[q];
#pragma unroll
                for (int i = 0; i < d; ++i)
#pragma unroll
                    for (int j = 0; j < d; ++j) y[i] -= A[(int64_t)q * d * d + i * d + j] * a[c * d + j];
            }
            T dz[d];
            apply_dinv<d, T>(dinv, u, y, dz);
#pragma unroll
            for (int i = 0; i < d; ++i) b[u * d + i] = a[u * d + i] + omega * dz[i];
        }
        __syncthreads();
        T* t = a; a = b; b = t;
    }
    if (a != z)
        for (int64_t i = threadIdx.x; i < n * d; i += blockDim.x) z[i] = a[i];
}

/* z = omega D^-1 r */
template <int d, typename T>
__global__ void k_amg_smooth0(int64_t n, const T* __restrict__ dinv, const T* __restrict__ r, T* __restrict__ z,
                              const double* __restrict__ omega_p, const DevScalars* ds)
{
    AMG_STOP;
    const T omega = (T)*omega_p;
    GRID_STRIDE(u, n)
    {
        T rv[d], zv[d];
#pragma unroll
        for (int i = 0; i < d; ++i) rv[i] = r[u * d + i];
        apply_dinv<d, T>(dinv, u, rv, zv);
#pragma unroll
        for (int i = 0; i < d; ++i) z[u * d + i] = omega * zv[i];
    }
}

/* zo = zi + omega D^-1 (r - A zi)   (zo != zi) */
template <int d, typename T>
__global__ void k_amg_jacobi(int64_t n, const int32_t* __restrict__ bptr, const int32_t* __restrict__ bcol,
                             const T* __restrict__ A, const T* __restrict__ dinv, const T* __restrict__ r,
                             const T* __restrict__ zi, T* __restrict__ zo, const double* __restrict__ omega_p,
                             const DevScalars* ds)
{
    AMG_STOP;
    const T omega = (T)*omega_p;
    GRID_STRIDE(u, n)
    {
        T y[d];
#pragma unroll
        for (int i = 0; i < d; ++i) y[i] = r[u * d + i];
        for (int32_t b = bptr[u]; b < bptr[u + 1]; ++b)
        {
            const int64_t c = bcol[b];
#pragma unroll
            for (int i = 0; i < d; ++i)
#pragma unroll
                for (int j = 0; j < d; ++j) y[i] -= A[(int64_t)b * d * d + i * d + j] * zi[c * d + j];
        }
        T dz[d];
        apply_dinv<d, T>(dinv, u, y, dz);
#pragma unroll
        for (int i = 0; i < d; ++i) zo[u * d + i] = zi[u * d + i] + omega * dz[i];
    }
}

/* t = r - A z, one block row per thread */
template <int d, typename T>
__global__ void k_amg_residual(int64_t n, const int32_t* __restrict__ bptr, const int32_t* __restrict__ bcol,
                               const T* __restrict__ A, const T* __restrict__ r, const T* __restrict__ z, T* __restrict__ t,
                               const DevScalars* ds)
{
    AMG_STOP;
    GRID_STRIDE(u, n)
    {
        T y[d];
#pragma unroll
        for (int i = 0; i < d; ++i) y[i] = r[u * d + i];
        for (int32_t b = bptr[u]; b < bptr[u + 1]; ++b)
        {
            const int64_t c = bcol[b];
#pragma unroll
            for (int i = 0; i < d; ++i)
#pragma unroll
                for (int j = 0; j < d; ++j) y[i] -= A[(int64_t)b * d * d + i * d + j] * z[c * d + j];
        }
#pragma unroll
        for (int i = 0; i < d; ++i) t[u * d + i] = y[i];
    }
}

/* rc[I] = sum of t over the aggregate I */
template <int d, typename T>
__global__ void k_amg_restrict(int64_t nc, const int32_t* __restrict__ aptr, const int32_t* __restrict__ aidx,
                               const T* __restrict__ t, T* __restrict__ rc, const DevScalars* ds)
{
    AMG_STOP;
    GRID_STRIDE(I, nc)
    {
        T acc[d];
#pragma unroll
        for (int i = 0; i < d; ++i) acc[i] = T(0);
        for (int32_t a = aptr[I]; a < aptr[I + 1]; ++a)
        {
            const int64_t u = aidx[a];
#pragma unroll
            for (int i = 0; i < d; ++i) acc[i] += t[u * d + i];
        }
#pragma unroll
        for (int i = 0; i < d; ++i) rc[I * d + i] = acc[i];
    }
}

/* one power-iteration step for rho(D^-1 A): y = D^-1 A (x / nx), ny = |y| */
template <int d, typename T>
__global__ void __launch_bounds__(RED_THREADS) k_amg_power(int64_t n, const int32_t* __restrict__ bptr,
                                                           const int32_t* __restrict__ bcol, const T* __restrict__ A,
                                                           const T* __restrict__ dinv, const T* __restrict__ x,
                                                           const double* __restrict__ nx, T* __restrict__ y, double* partials,
                                                           unsigned* counter, double* ny)
{
    const T scale = (T)(1.0 / *nx);
    double part[1] = {0.0};
    GRID_STRIDE(u, n)
    {
        T v[d];
#pragma unroll
        for (int i = 0; i < d; ++i) v[i] = T(0);
        for (int32_t b = bptr[u]; b < bptr[u + 1]; ++b)
        {
            const int64_t c = bcol[b];
#pragma unroll
            for (int i = 0; i < d; ++i)
#pragma unroll
                for (int j = 0; j < d; ++j) v[i] += A[(int64_t)b * d * d + i * d + j] * (x[c * d + j] * scale);
        }
        T o[d];
        apply_dinv<d, T>(dinv, u, v, o);
#pragma unroll
        for (int i = 0; i < d; ++i)
        {
            y[u * d + i] = o[i];
            part[0] += (double)(o[i] * o[i]);
        }
    }
    double tot[1];
    if (!grid_sum<1>(part, partials, counter, tot)) return;
    if (threadIdx.x == 0) *ny = sqrt(tot[0]) > 0.0 ? sqrt(tot[0]) : 1.0;
}

/* start vector of the power iteration (a fixed pseudo-random pattern) */
template <typename T>
__global__ void k_amg_power_start(int64_t m, T* x, double* nx)
{
    GRID_STRIDE(i, m)
    {
        uint32_t h = (uint32_t)i * 2654435761u;
        h ^= h >> 15;
        x[i] = (T)(0.5 + (double)(h & 0xffff) / 65536.0);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *nx = 1.0;
}

/* omega = factor / rho from the last two power-iteration norms */
__global__ void k_amg_set_omega(const double* ny, double* omega)
{
    const double rho = *ny;
    *omega = (rho > 0.0 && isfinite(rho)) ? AMG_OMEGA_FACTOR / rho : 0.5;
}

/* z[u] += zc[agg[u]] */
template <int d, typename T>
__global__ void k_amg_prolong(int64_t n, const int32_t* __restrict__ agg, const T* __restrict__ zc, T* __restrict__ z,
                              const DevScalars* ds)
{
    AMG_STOP;
    GRID_STRIDE(u, n)
    {
        const int64_t I = agg[u];
#pragma unroll
        for (int i = 0; i < d; ++i) z[u * d + i] += zc[I * d + i];
    }
}

/* ---- host launchers ------------------------------------------------------------- */
/* a grid for n rows: enough blocks to cover them once, at most the reduction grid */
static unsigned grid_for(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(RED_BLOCKS, (n + RED_THREADS - 1) / RED_THREADS)); }
template <int d, typename T>
static void vcycle(Problem& P, size_t l, const T* r, T* out)
{
    cudaStream_t s = P.stream;
    AmgLevel& L = P.amg[l];
    const T* A = l == 0 ? (const T*)P.H : (const T*)L.A;
    const T* dinv = (const T*)L.dinv;
    const double* om = P.amg_omega + l;
    T* w = (T*)L.w;
    const DevScalars* ds = P.ds;
    if (l + 1 == P.amg.size())
    {
        k_amg_coarse<d, T><<<1, AMG_COARSE_THREADS, 0, s>>>(L.n, L.bptr, L.bcol, A, dinv, r, out, w, om, ds);
        P.n_launches += 1;
        return;
    }
    AmgLevel& C = P.amg[l + 1];
    const unsigned g = grid_for(L.n), gc = grid_for(C.n);
    k_amg_smooth0<d, T><<<g, RED_THREADS, 0, s>>>(L.n, dinv, r, w, om, ds);
    k_amg_residual<d, T><<<g, RED_THREADS, 0, s>>>(L.n, L.bptr, L.bcol, A, r, w, (T*)L.t, ds);
    k_amg_restrict<d, T><<<gc, RED_THREADS, 0, s>>>(C.n, C.aptr, C.aidx, (const T*)L.t, (T*)C.r, ds);
    P.n_launches += 3;
    vcycle<d, T>(P, l + 1, (const T*)C.r, (T*)C.z);
    k_amg_prolong<d, T><<<g, RED_THREADS, 0, s>>>(L.n, C.agg, (const T*)C.z, w, ds);
    k_amg_jacobi<d, T><<<g, RED_THREADS, 0, s>>>(L.n, L.bptr, L.bcol, A, dinv, r, w, out, om, ds);
    P.n_launches += 2;
}

template <int d, typename T>
static void values(Problem& P)
{
    cudaStream_t s = P.stream;
    for (size_t l = 0; l < P.amg.size(); ++l)
    {
        AmgLevel& L = P.amg[l];
        const T* A = l == 0 ? (const T*)P.H : (const T*)L.A;
        if (l > 0)
        {
            const T* Af = l == 1 ? (const T*)P.H : (const T*)P.amg[l - 1].A;
            k_amg_galerkin<d, T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(L.nb, L.cptr, L.cidx, Af, (T*)L.A);
        }
        k_diag_inv<d, T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(L.n, L.diag, A, 0.0, (T*)L.dinv);
        // rho(D^-1 A) by power iteration (z, w as scratch), then the damping
        const unsigned g = grid_for(L.n);
        double* nrm = P.amg_omega + AMG_MAX_LEVELS;   // two norms of scratch
        k_amg_power_start<T><<<g, RED_THREADS, 0, s>>>(L.n * d, (T*)L.z, nrm);
        T* a = (T*)L.z;
        T* b = (T*)L.w;
        for (int k = 0; k < AMG_POWER_STEPS; ++k)
        {
            k_amg_power<d, T><<<g, RED_THREADS, 0, s>>>(L.n, L.bptr, L.bcol, A, (const T*)L.dinv, a, nrm + (k & 1), b,
                                                        P.partials, P.counters + 10, nrm + ((k + 1) & 1));
            std::swap(a, b);
        }
        k_amg_set_omega<<<1, 1, 0, s>>>(nrm + (AMG_POWER_STEPS & 1), P.amg_omega + l);
        P.n_launches += (l > 0 ? 2 : 1) + 2 + AMG_POWER_STEPS;
    }
}

tad_status amg_prepare(Problem& P, int precision)
{
    tad_status st = amg_build(P);
    if (st != TAD_OK) return st;
    const bool f32 = precision == TAD_PREC_MIXED;
    switch (P.d)
    {
    case 1: f32 ? values<1, float>(P) : values<1, double>(P); break;
    case 2: f32 ? values<2, float>(P) : values<2, double>(P); break;
    default: f32 ? values<3, float>(P) : values<3, double>(P); break;
    }
    TAD_CUDA_TRY(cudaGetLastError());
    return TAD_OK;
}

void amg_vcycle(Problem& P, int precision, const void* r, void* z)
{
    const bool f32 = precision == TAD_PREC_MIXED;
    switch (P.d)
    {
    case 1: f32 ? vcycle<1, float>(P, 0, (const float*)r, (float*)z) : vcycle<1, double>(P, 0, (const double*)r, (double*)z); break;
    case 2: f32 ? vcycle<2, float>(P, 0, (const float*)r, (float*)z) : vcycle<2, double>(P, 0, (const double*)r, (double*)z); break;
    default: f32 ? vcycle<3, float>(P, 0, (const float*)r, (float*)z) : vcycle<3, double>(P, 0, (const double*)r, (double*)z); break;
    }
}

int amg_levels(const Problem& P) { return (int)P.amg.size(); }

} // namespace tadlib
