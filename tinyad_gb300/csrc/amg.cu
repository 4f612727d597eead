/*
 * Smoothed-aggregation AMG preconditioner for the device PCG.
 *
 * Block-Jacobi PCG needs O(sqrt(cond)) iterations: on the 1.64M-face disk
 * the late Newton steps take 200-850 of them at a 1e-2 relative residual,
 * and those steps are nearly all of a solve's time.  Conjugate gradients
 * preconditioned by one V-cycle of this hierarchy take 10-20.
 *
 * Hierarchy, per level l (d x d blocks on every level):
 *   aggregation  greedy one-ring aggregates of the block graph (a row whose
 *                neighbours are all free roots an aggregate of its one-ring;
 *                rows left over join the aggregate of their first aggregated
 *                neighbour; isolated rows are their own aggregate);
 *   P_t          tentative prolongation of the d translations: the block of
 *                fine row u in column agg(u) is I / sqrt(|agg(u)|) (the
 *                orthonormal basis of the translations on the aggregate);
 *   P            smoothed prolongation P = (I - omega S A) P_t, S the l1
 *                block-Jacobi inverse below and omega = AMG_PROLONG_OMEGA;
 *   Q            Q = A P, kept for the V-cycle's fused post-smoothing;
 *   A_c          the Galerkin product P^T Q, the next level's matrix.
 * The sparsity patterns (aggregates, P, Q, A_c and the transposed lists of
 * P) are built once per problem on the host; the values are recomputed on
 * the device for every Hessian, each output row by one thread in a fixed
 * order (deterministic, no atomics).
 *
 * V-cycle (symmetric positive definite for a symmetric positive definite A,
 * so CG stays valid), per level with the l1 block-Jacobi smoother
 * S = (A_uu + diag(sum_{v != u} |A_uv| row sums))^-1, which converges
 * without a damping estimate:
 *   x = S r                         (pre-smoothing from zero; fused into the
 *                                    kernel that produces r)
 *   res = r - A x                   (k_amg_residual)
 *   r_c = P^T res, x_c = S_c r_c    (k_amg_restrict, one thread per coarse row)
 *   x_c <- V-cycle of the next level
 *   x += P x_c + S (res - Q x_c)    (k_amg_post, as x += R x_c + S res with
 *                                    R = P - S Q formed with Q: prolongation and
 *                                    post-smoothing in one pass, since
 *                                    r - A (x + P x_c) = res - Q x_c)
 * and on the coarsest level (<= AMG_COARSE_ROWS block rows) AMG_COARSE_SWEEPS
 * l1 block-Jacobi sweeps in one thread block.  All kernels return at once
 * when the PCG's stop flag is set, so chunks of iterations are captured in a
 * CUDA graph.  Values and vectors are in the PCG's precision.
 */
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.hh"
#include "grid_reduce.cuh"
#include "bsr_kernels.cuh"

namespace tadlib {

constexpr int64_t AMG_COARSE_ROWS = 256;
constexpr int AMG_MAX_LEVELS = 12;
constexpr int AMG_COARSE_SWEEPS = 12;
constexpr int AMG_COARSE_THREADS = 1024;
/* damping of the prolongator smoother I - omega S A, S the l1 block-Jacobi
   inverse: rho(S A) <= 1 for symmetric positive definite A, so omega < 2
   keeps it stable without a spectral-radius estimate (the usual 4 / (3 rho)
   with rho(D^-1 A) from power iterations took as many PCG iterations on the
   disk parametrisations and 8 extra SpMVs per level and Hessian) */
constexpr double AMG_PROLONG_OMEGA = 1.8;
/* warp-cooperative setup kernels keep one coarse row's accumulators in
   shared memory: rows up to this many blocks (longer: a thread per row) */
constexpr int AMG_ROW_CAP = 96;
constexpr int AMG_SETUP_WARPS = 4;   // warps per block of the setup kernels
/* prolongator rows of at most this many blocks are summed in registers (2D
   rows have up to ~9; 3D rows 10-30, which keep the memory path) */
template <int d> struct ProlongRegs { static constexpr int value = d <= 2 ? 8 : 1; };

/* ---- host: aggregation and the patterns of P, Q, A_c ----------------------- */
namespace {

struct HostLevel
{
    int64_t n = 0;
    std::vector<int32_t> bptr, bcol, diag;   // A_l
    // transfer to the next level (all but the coarsest)
    int64_t nc = 0;
    std::vector<int32_t> agg;                // fine row -> aggregate (coarse row)
    std::vector<double> cscale;              // per aggregate: 1 / sqrt(size)
    std::vector<int32_t> pptr, pcol;         // P: fine rows x aggregates
    std::vector<int32_t> pslot;              // per block of A_l: the P block it feeds in the smoothing
    std::vector<int32_t> pdiag;              // per fine row: its P block in column agg(u)
    std::vector<int32_t> qptr, qcol;         // Q = A_l P
    std::vector<int32_t> qlptr, qla, qlp;    // per Q block: its (A block, P block) products
    std::vector<int32_t> qrow, qpb;          // per Q block: its row, and the P block at its position (-1: none)
    std::vector<int32_t> tptr, tu, tp;       // per aggregate: (fine row, P block) with P(u, I) != 0, by u
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

/* rows of a CSR pattern, each the sorted unique list fill(u, out) produces;
   two passes (count, then write), rows in parallel */
template <typename F>
void build_rows(int64_t n, std::vector<int32_t>& ptr, std::vector<int32_t>& col, F fill)
{
    ptr.assign(n + 1, 0);
#pragma omp parallel
    {
        std::vector<int32_t> tmp;
#pragma omp for schedule(dynamic, 1024)
        for (int64_t u = 0; u < n; ++u)
        {
            tmp.clear();
            fill(u, tmp);
            std::sort(tmp.begin(), tmp.end());
            ptr[u + 1] = (int32_t)(std::unique(tmp.begin(), tmp.end()) - tmp.begin());
        }
    }
    for (int64_t u = 0; u < n; ++u) ptr[u + 1] += ptr[u];
    col.resize(ptr[n]);
#pragma omp parallel
    {
        std::vector<int32_t> tmp;
#pragma omp for schedule(dynamic, 1024)
        for (int64_t u = 0; u < n; ++u)
        {
            tmp.clear();
            fill(u, tmp);
            std::sort(tmp.begin(), tmp.end());
            tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
            std::copy(tmp.begin(), tmp.end(), col.begin() + ptr[u]);
        }
    }
}

int32_t find_in(const std::vector<int32_t>& col, int32_t b, int32_t e, int32_t key)
{
    const auto it = std::lower_bound(col.begin() + b, col.begin() + e, key);
    return (it != col.begin() + e && *it == key) ? (int32_t)(it - col.begin()) : -1;
}

/* the transfer of level F to the next level C (F's agg / nc set) */
void transfer(HostLevel& F, HostLevel& C)
{
    const int64_t n = F.n, nc = F.nc;
    std::vector<int32_t> size(nc, 0);
    for (int64_t u = 0; u < n; ++u) ++size[F.agg[u]];
    F.cscale.resize(nc);
    for (int64_t I = 0; I < nc; ++I) F.cscale[I] = 1.0 / std::sqrt((double)std::max(1, size[I]));
    // P: the aggregates of the one-ring (and of u itself)
    build_rows(n, F.pptr, F.pcol, [&](int64_t u, std::vector<int32_t>& out) {
        out.push_back(F.agg[u]);
        for (int32_t q = F.bptr[u]; q < F.bptr[u + 1]; ++q) out.push_back(F.agg[F.bcol[q]]);
    });
    F.pslot.resize(F.bcol.size());
    F.pdiag.resize(n);
#pragma omp parallel for schedule(static)
    for (int64_t u = 0; u < n; ++u)
    {
        for (int32_t q = F.bptr[u]; q < F.bptr[u + 1]; ++q) F.pslot[q] = find_in(F.pcol, F.pptr[u], F.pptr[u + 1], F.agg[F.bcol[q]]);
        F.pdiag[u] = find_in(F.pcol, F.pptr[u], F.pptr[u + 1], F.agg[u]);
    }
    // Q = A P: the P columns of the neighbours
    build_rows(n, F.qptr, F.qcol, [&](int64_t u, std::vector<int32_t>& out) {
        for (int32_t q = F.bptr[u]; q < F.bptr[u + 1]; ++q)
        {
            const int32_t v = F.bcol[q];
            out.insert(out.end(), F.pcol.begin() + F.pptr[v], F.pcol.begin() + F.pptr[v + 1]);
        }
    });
    // per Q block: its row and the P block at the same (row, column), for R = P - S Q
    F.qrow.resize(F.qcol.size());
    F.qpb.resize(F.qcol.size());
#pragma omp parallel for schedule(static)
    for (int64_t u = 0; u < n; ++u)
        for (int32_t b = F.qptr[u]; b < F.qptr[u + 1]; ++b)
        {
            F.qrow[b] = (int32_t)u;
            F.qpb[b] = find_in(F.pcol, F.pptr[u], F.pptr[u + 1], F.qcol[b]);
        }
    // the products of each Q block: (A block, P block) pairs in row order of A, then of P
    {
        std::vector<int32_t> cnt(F.qcol.size() + 1, 0);
#pragma omp parallel for schedule(dynamic, 1024)
        for (int64_t u = 0; u < n; ++u)
            for (int32_t a = F.bptr[u]; a < F.bptr[u + 1]; ++a)
            {
                const int32_t v = F.bcol[a];
                for (int32_t p = F.pptr[v]; p < F.pptr[v + 1]; ++p)
                    ++cnt[find_in(F.qcol, F.qptr[u], F.qptr[u + 1], F.pcol[p]) + 1];   // rows are disjoint: no race
            }
        for (size_t b = 0; b < F.qcol.size(); ++b) cnt[b + 1] += cnt[b];
        F.qlptr = cnt;
        F.qla.resize(cnt.back());
        F.qlp.resize(cnt.back());
#pragma omp parallel for schedule(dynamic, 1024)
        for (int64_t u = 0; u < n; ++u)
        {
            for (int32_t a = F.bptr[u]; a < F.bptr[u + 1]; ++a)
            {
                const int32_t v = F.bcol[a];
                for (int32_t p = F.pptr[v]; p < F.pptr[v + 1]; ++p)
                {
                    const int32_t b = find_in(F.qcol, F.qptr[u], F.qptr[u + 1], F.pcol[p]);
                    const int32_t k = cnt[b]++;
                    F.qla[k] = a;
                    F.qlp[k] = p;
                }
            }
        }
    }
    // transposed P: per aggregate, the (fine row, P block) pairs in fine row order
    F.tptr.assign(nc + 1, 0);
    for (size_t p = 0; p < F.pcol.size(); ++p) ++F.tptr[F.pcol[p] + 1];
    for (int64_t I = 0; I < nc; ++I) F.tptr[I + 1] += F.tptr[I];
    F.tu.resize(F.pcol.size());
    F.tp.resize(F.pcol.size());
    {
        std::vector<int32_t> fill(F.tptr.begin(), F.tptr.end() - 1);
        for (int64_t u = 0; u < n; ++u)
            for (int32_t p = F.pptr[u]; p < F.pptr[u + 1]; ++p)
            {
                const int32_t t = fill[F.pcol[p]]++;
                F.tu[t] = (int32_t)u;
                F.tp[t] = p;
            }
    }
    // A_c = P^T Q: the Q columns of the rows in each aggregate's support
    C.n = nc;
    build_rows(nc, C.bptr, C.bcol, [&](int64_t I, std::vector<int32_t>& out) {
        out.push_back((int32_t)I);
        for (int32_t t = F.tptr[I]; t < F.tptr[I + 1]; ++t)
        {
            const int32_t u = F.tu[t];
            out.insert(out.end(), F.qcol.begin() + F.qptr[u], F.qcol.begin() + F.qptr[u + 1]);
        }
    });
    C.diag.resize(nc);
    for (int64_t I = 0; I < nc; ++I) C.diag[I] = find_in(C.bcol, C.bptr[I], C.bptr[I + 1], (int32_t)I);
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
        for (void* q : {(void*)L.pptr, (void*)L.pcol, (void*)L.pslot, (void*)L.pdiag, (void*)L.qptr, (void*)L.qcol,
                        (void*)L.tptr, (void*)L.tu, (void*)L.tp, (void*)L.cscale, (void*)L.qlptr, (void*)L.qla,
                        (void*)L.qlp, (void*)L.qrow, (void*)L.qpb, L.Pv, L.Qv, L.Rv, L.dl1, L.r, L.x, L.res, L.w})
            if (q) cudaFree(q);
    }
    P.amg.clear();
    P.amg_values_ready = false;
}

/* pattern-level hierarchy (once per problem) */
tad_status amg_build(Problem& P)
{
    if (!P.amg.empty()) return TAD_OK;
    const int d = P.d;
    std::vector<HostLevel> H(1);
    H[0].n = P.n_handles;
    H[0].bptr.assign(P.bptr_h.begin(), P.bptr_h.end());
    H[0].bcol.assign(P.bcol_h.begin(), P.bcol_h.end());
    while ((int)H.size() < AMG_MAX_LEVELS && H.back().n > AMG_COARSE_ROWS)
    {
        HostLevel& F = H.back();
        int64_t nc = 0;
        std::vector<int32_t> agg = aggregate(F.n, F.bptr, F.bcol, nc);
        if (nc >= F.n * 9 / 10) break;   // coarsening stalled
        F.agg = std::move(agg);
        F.nc = nc;
        HostLevel C;
        transfer(F, C);
        H.push_back(std::move(C));
    }
    P.amg.resize(H.size());
    const size_t vb = sizeof(double);   // values and vectors sized for FP64, used as T
    const size_t bs = (size_t)d * d * vb;
    auto fail = [&]() { amg_free(P); return amg_fail("AMG: device allocation failed"); };
    for (size_t l = 0; l < H.size(); ++l)
    {
        AmgLevel& L = P.amg[l];
        HostLevel& h = H[l];
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
                upload(&L.diag, h.diag) != cudaSuccess || cudaMalloc(&L.A, std::max<int64_t>(L.nb, 1) * bs) != cudaSuccess)
                return fail();
        }
        const size_t nv = (size_t)std::max<int64_t>(L.n, 1) * d * vb;
        if (cudaMalloc(&L.dl1, std::max<int64_t>(L.n, 1) * bs) != cudaSuccess || cudaMalloc(&L.r, nv) != cudaSuccess ||
            cudaMalloc(&L.x, nv) != cudaSuccess || cudaMalloc(&L.res, nv) != cudaSuccess || cudaMalloc(&L.w, nv) != cudaSuccess)
            return fail();
        L.max_row = 0;
        for (int64_t u = 0; u < h.n; ++u) L.max_row = std::max<int64_t>(L.max_row, h.bptr[u + 1] - h.bptr[u]);
        if (l + 1 < H.size())
        {
            L.nc = h.nc;
            L.np = (int64_t)h.pcol.size();
            L.nq = (int64_t)h.qcol.size();
            if (upload(&L.pptr, h.pptr) != cudaSuccess || upload(&L.pcol, h.pcol) != cudaSuccess ||
                upload(&L.pslot, h.pslot) != cudaSuccess || upload(&L.pdiag, h.pdiag) != cudaSuccess ||
                upload(&L.qptr, h.qptr) != cudaSuccess || upload(&L.qcol, h.qcol) != cudaSuccess ||
                upload(&L.tptr, h.tptr) != cudaSuccess || upload(&L.tu, h.tu) != cudaSuccess ||
                upload(&L.tp, h.tp) != cudaSuccess || upload(&L.cscale, h.cscale) != cudaSuccess ||
                upload(&L.qlptr, h.qlptr) != cudaSuccess || upload(&L.qla, h.qla) != cudaSuccess ||
                upload(&L.qlp, h.qlp) != cudaSuccess || upload(&L.qrow, h.qrow) != cudaSuccess ||
                upload(&L.qpb, h.qpb) != cudaSuccess ||
                cudaMalloc(&L.Pv, std::max<int64_t>(L.np, 1) * bs) != cudaSuccess ||
                cudaMalloc(&L.Qv, std::max<int64_t>(L.nq, 1) * bs) != cudaSuccess ||
                cudaMalloc(&L.Rv, std::max<int64_t>(L.nq, 1) * bs) != cudaSuccess)
                return fail();
        }
    }
    P.amg_values_ready = false;
    return TAD_OK;
}

/* ---- device kernels ---------------------------------------------------------- */
#define AMG_STOP if (ds && *(volatile const int32_t*)&ds->done) return

template <int d, typename T>
__device__ __forceinline__ void mat_mul_acc(const T (&a)[d * d], const T (&b)[d * d], T* __restrict__ c)
{
#pragma unroll
    for (int i = 0; i < d; ++i)
#pragma unroll
        for (int j = 0; j < d; ++j)
        {
            T s = c[i * d + j];
#pragma unroll
            for (int k = 0; k < d; ++k) s += a[i * d + k] * b[k * d + j];
            c[i * d + j] = s;
        }
}

/* inverse of a d x d matrix (symmetric positive definite expected); a
   non-positive determinant falls back to the inverse of the positive diagonal */
template <int d, typename T>
__device__ __forceinline__ void small_inverse(const T (&A)[d * d], T (&I)[d * d])
{
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
    if (!(det > T(0) && isfinite(det)))
    {
#pragma unroll
        for (int i = 0; i < d; ++i)
#pragma unroll
            for (int j = 0; j < d; ++j)
                I[i * d + j] = (i == j && A[i * d + i] > T(0)) ? T(1) / A[i * d + i] : (i == j ? T(1) : T(0));
    }
}

/* per row: the inverted l1 block -- the diagonal block plus, on its
   diagonal, the absolute row sums of the off-diagonal blocks */
template <int d, typename T>
__global__ void k_amg_diag(int64_t n, const int32_t* __restrict__ bptr, const int32_t* __restrict__ bcol,
                           const int32_t* __restrict__ diag, const T* __restrict__ A, T* __restrict__ dl1)
{
    GRID_STRIDE(u, n)
    {
        T D[d * d], off[d];
#pragma unroll
        for (int i = 0; i < d * d; ++i) D[i] = T(0);
#pragma unroll
        for (int i = 0; i < d; ++i) off[i] = T(0);
        const int32_t db = diag[u];
        for (int32_t q = bptr[u]; q < bptr[u + 1]; ++q)
        {
            T B[d * d];
            load_block<d, T>(A + (int64_t)q * d * d, B);
            if (q == db)
            {
#pragma unroll
                for (int i = 0; i < d * d; ++i) D[i] = B[i];
            }
            else
            {
#pragma unroll
                for (int i = 0; i < d; ++i)
#pragma unroll
                    for (int j = 0; j < d; ++j) off[i] += fabs(B[i * d + j]);
            }
        }
#pragma unroll
        for (int i = 0; i < d; ++i) D[i * d + i] += off[i];
        T I[d * d];
        small_inverse<d, T>(D, I);
#pragma unroll
        for (int i = 0; i < d * d; ++i) dl1[u * d * d + i] = I[i];
    }
}

/* P = (I - omega S A) P_t, one thread per fine row: the blocks of A are
   summed per aggregate of their column (in row order), then
   P(u, J) = [J == agg(u)] c_J I - omega c_J S_u Sum(u, J), c_J = 1/sqrt|J| */
template <int d, typename T>
__global__ void k_amg_prolongator(int64_t n, const int32_t* __restrict__ bptr, const int32_t* __restrict__ pslot,
                                  const int32_t* __restrict__ pptr, const int32_t* __restrict__ pcol,
                                  const int32_t* __restrict__ pdiag, const double* __restrict__ cscale,
                                  const T* __restrict__ A, const T* __restrict__ dl1, T* __restrict__ Pv)
{
    const T omega = (T)AMG_PROLONG_OMEGA;
    constexpr int R = ProlongRegs<d>::value;
    GRID_STRIDE(u, n)
    {
        const int32_t p0 = pptr[u], p1 = pptr[u + 1];
        if (p1 - p0 <= R)
        {
            // the row's (A S-weighted) sums in registers: S[k] = sum of the A blocks
            // feeding P block p0 + k, in row order (the slot picked by a compare
            // chain, not a register index)
            T S[R][d * d];
#pragma unroll
            for (int k = 0; k < R; ++k)
#pragma unroll
                for (int i = 0; i < d * d; ++i) S[k][i] = T(0);
            for (int32_t q = bptr[u]; q < bptr[u + 1]; ++q)
            {
                T B[d * d];
                load_block<d, T>(A + (int64_t)q * d * d, B);
                const int32_t k = pslot[q] - p0;
#pragma unroll
                for (int kk = 0; kk < R; ++kk)
                    if (kk == k)
#pragma unroll
                        for (int i = 0; i < d * d; ++i) S[kk][i] += B[i];
            }
            T Di[d * d];
            load_block<d, T>(dl1 + u * d * d, Di);
            const int32_t pd = pdiag[u];
#pragma unroll
            for (int kk = 0; kk < R; ++kk)
            {
                const int32_t p = p0 + kk;
                if (p >= p1) break;
                const T c = (T)cscale[pcol[p]];
                T O[d * d];
#pragma unroll
                for (int i = 0; i < d * d; ++i) O[i] = T(0);
                mat_mul_acc<d, T>(Di, S[kk], O);
#pragma unroll
                for (int i = 0; i < d; ++i)
#pragma unroll
                    for (int j = 0; j < d; ++j)
                        Pv[(int64_t)p * d * d + i * d + j] = ((p == pd && i == j) ? c : T(0)) - omega * c * O[i * d + j];
            }
            continue;
        }
        for (int64_t i = (int64_t)p0 * d * d; i < (int64_t)p1 * d * d; ++i) Pv[i] = T(0);
        for (int32_t q = bptr[u]; q < bptr[u + 1]; ++q)
        {
            T B[d * d];
            load_block<d, T>(A + (int64_t)q * d * d, B);
            T* S = Pv + (int64_t)pslot[q] * d * d;
#pragma unroll
            for (int i = 0; i < d * d; ++i) S[i] += B[i];
        }
        T Di[d * d];
#pragma unroll
        for (int i = 0; i < d * d; ++i) Di[i] = dl1[u * d * d + i];
        const int32_t pd = pdiag[u];
        for (int32_t p = p0; p < p1; ++p)
        {
            const T c = (T)cscale[pcol[p]];
            T S[d * d], O[d * d];
#pragma unroll
            for (int i = 0; i < d * d; ++i) { S[i] = Pv[(int64_t)p * d * d + i]; O[i] = T(0); }
            mat_mul_acc<d, T>(Di, S, O);
#pragma unroll
            for (int i = 0; i < d; ++i)
#pragma unroll
                for (int j = 0; j < d; ++j)
                    Pv[(int64_t)p * d * d + i * d + j] = ((p == pd && i == j) ? c : T(0)) - omega * c * O[i * d + j];
        }
    }
}

/* first index in col[b, e) equal to key (the column is there by construction) */
__device__ __forceinline__ int32_t find_col(const int32_t* __restrict__ col, int32_t b, int32_t e, int32_t key)
{
    while (e - b > 4)
    {
        const int32_t m = (b + e) >> 1;
        if (col[m] <= key) b = m;
        else e = m;
    }
    for (; b < e; ++b)
        if (col[b] == key) return b;
    return -1;
}

/* Q = A P, one thread per Q block: the sum of its (A block, P block)
   products in the list's fixed order; and R = P - S Q on the same block
   (S the l1 inverse of the block's row; P's block at that position where P
   has one -- its row pattern lies in Q's for every row with a diagonal block,
   and a row without one is a variable no element uses, whose residual stays
   zero), the post-smoothing's operator: x += P x_c + S (res - Q x_c) is
   x += R x_c + S res, one row product instead of two in every V-cycle */
template <int d, typename T>
__global__ void k_amg_q(int64_t nq, const int32_t* __restrict__ qlptr, const int32_t* __restrict__ qla,
                        const int32_t* __restrict__ qlp, const int32_t* __restrict__ qrow, const int32_t* __restrict__ qpb,
                        const T* __restrict__ A, const T* __restrict__ Pv, const T* __restrict__ dl1, T* __restrict__ Qv,
                        T* __restrict__ Rv)
{
    GRID_STRIDE(b, nq)
    {
        T acc[d * d];
#pragma unroll
        for (int i = 0; i < d * d; ++i) acc[i] = T(0);
        const int32_t k1 = qlptr[b + 1];
        for (int32_t k = qlptr[b]; k < k1; ++k)
        {
            T B[d * d], Pb[d * d];
            load_block<d, T>(A + (int64_t)__ldg(qla + k) * d * d, B);
            load_block<d, T>(Pv + (int64_t)__ldg(qlp + k) * d * d, Pb);
            mat_mul_acc<d, T>(B, Pb, acc);
        }
        T S[d * d], R[d * d];
        load_block<d, T>(dl1 + (int64_t)qrow[b] * d * d, S);
        const int32_t pb = qpb[b];
        if (pb >= 0) load_block<d, T>(Pv + (int64_t)pb * d * d, R);
        else
#pragma unroll
            for (int i = 0; i < d * d; ++i) R[i] = T(0);
        T O[d * d];
#pragma unroll
        for (int i = 0; i < d * d; ++i) O[i] = T(0);
        mat_mul_acc<d, T>(S, acc, O);
#pragma unroll
        for (int i = 0; i < d * d; ++i) R[i] -= O[i];
        if constexpr (d == 2 && sizeof(T) == 4)
        {
            reinterpret_cast<float4*>(Qv)[b] = make_float4(acc[0], acc[1], acc[2], acc[3]);
            reinterpret_cast<float4*>(Rv)[b] = make_float4(R[0], R[1], R[2], R[3]);
        }
        else
        {
#pragma unroll
            for (int i = 0; i < d * d; ++i) { Qv[b * d * d + i] = acc[i]; Rv[b * d * d + i] = R[i]; }
        }
    }
}

/* slot of key in the sorted col[0, m) (shared memory; the key is there by construction) */
__device__ __forceinline__ int32_t find_slot(const int32_t* col, int32_t m, int32_t key)
{
    int32_t b = 0, e = m;
    while (e - b > 1)
    {
        const int32_t h = (b + e) >> 1;
        if (col[h] <= key) b = h;
        else e = h;
    }
    return (m > 0 && col[b] == key) ? b : -1;
}

/* groups per warp of k_amg_galerkin (each with its own accumulators in
   shared memory): 4 for blocks of up to 16 bytes, 2 up to 36, else 1 */
template <int d, typename T> struct GalerkinGroups
{
    static constexpr int value = (d * d * (int)sizeof(T) <= 16) ? 4 : (d * d * (int)sizeof(T) <= 36) ? 2 : 1;
};

/* A_c = P^T Q, one warp per coarse row I (rows of at most AMG_ROW_CAP
   blocks).  The warp is split into G groups; group g takes the pairs
   (u, P(u, I)) number g, g + G, ... of the row's list, and its lanes take the
   blocks Q(u, J) of row u, whose columns are distinct, into the group's own
   accumulators in shared memory -- so no two lanes add into one accumulator
   at once, and each accumulator sums its pairs in list order.  The G partial
   rows are added in group order at the end: a fixed order, no atomics.  (One
   group of 32 lanes left most lanes idle on rows of 7-12 Q blocks and walked
   the list's dependent loads one pair at a time.) */
template <int d, typename T>
__global__ void __launch_bounds__(AMG_SETUP_WARPS * 32) k_amg_galerkin(int64_t nc, const int32_t* __restrict__ tptr,
                                                                       const int32_t* __restrict__ tu,
                                                                       const int32_t* __restrict__ tp, const T* __restrict__ Pv,
                                                                       const int32_t* __restrict__ qptr,
                                                                       const int32_t* __restrict__ qcol,
                                                                       const T* __restrict__ Qv, const int32_t* __restrict__ cptr,
                                                                       const int32_t* __restrict__ ccol, T* __restrict__ Ac)
{
    constexpr int G = GalerkinGroups<d, T>::value, LG = 32 / G;
    __shared__ T acc_s[AMG_SETUP_WARPS][G][AMG_ROW_CAP * d * d];
    __shared__ int32_t col_s[AMG_SETUP_WARPS][AMG_ROW_CAP];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane / LG, gl = lane % LG;
    int32_t* col = col_s[w];
    T* acc = acc_s[w][g];
    for (int64_t I = blockIdx.x * (int64_t)AMG_SETUP_WARPS + w; I < nc; I += (int64_t)gridDim.x * AMG_SETUP_WARPS)
    {
        const int32_t c0 = cptr[I], m = cptr[I + 1] - c0;
        for (int32_t k = lane; k < m; k += 32) col[k] = ccol[c0 + k];
        for (int32_t k = gl; k < m; k += LG)
#pragma unroll
            for (int i = 0; i < d * d; ++i) acc[k * d * d + i] = T(0);
        __syncwarp();
        const int32_t t_end = tptr[I + 1];
        for (int32_t tb = tptr[I]; tb < t_end; tb += G)
        {
            const int32_t t = tb + g;
            if (t < t_end)
            {
                const int32_t u = tu[t];
                T Pt[d * d];
                {
                    T Pb[d * d];
                    load_block<d, T>(Pv + (int64_t)tp[t] * d * d, Pb);
#pragma unroll
                    for (int i = 0; i < d; ++i)
#pragma unroll
                        for (int j = 0; j < d; ++j) Pt[i * d + j] = Pb[j * d + i];
                }
                const int32_t q1 = qptr[u + 1];
                for (int32_t q = qptr[u] + gl; q < q1; q += LG)
                {
                    T Qb[d * d];
                    load_block<d, T>(Qv + (int64_t)q * d * d, Qb);
                    const int32_t sl = find_slot(col, m, qcol[q]);
                    if (sl >= 0) mat_mul_acc<d, T>(Pt, Qb, acc + sl * d * d);
                }
            }
            __syncwarp();
        }
        for (int32_t k = lane; k < m; k += 32)
        {
#pragma unroll
            for (int i = 0; i < d * d; ++i)
            {
                T v = acc_s[w][0][k * d * d + i];
#pragma unroll
                for (int h = 1; h < G; ++h) v += acc_s[w][h][k * d * d + i];
                Ac[(int64_t)(c0 + k) * d * d + i] = v;
            }
        }
        __syncwarp();
    }
}

/* the same, one thread per coarse row, for hierarchies with a coarse row
   longer than AMG_ROW_CAP blocks (accumulating in the output row) */
template <int d, typename T>
__global__ void k_amg_galerkin_rows(int64_t nc, const int32_t* __restrict__ tptr, const int32_t* __restrict__ tu,
                                    const int32_t* __restrict__ tp, const T* __restrict__ Pv, const int32_t* __restrict__ qptr,
                                    const int32_t* __restrict__ qcol, const T* __restrict__ Qv, const int32_t* __restrict__ cptr,
                                    const int32_t* __restrict__ ccol, T* __restrict__ Ac)
{
    GRID_STRIDE(I, nc)
    {
        const int32_t c0 = cptr[I], c1 = cptr[I + 1];
        for (int64_t i = (int64_t)c0 * d * d; i < (int64_t)c1 * d * d; ++i) Ac[i] = T(0);
        for (int32_t t = tptr[I]; t < tptr[I + 1]; ++t)
        {
            const int32_t u = tu[t];
            T Pt[d * d];
            {
                T Pb[d * d];
                load_block<d, T>(Pv + (int64_t)tp[t] * d * d, Pb);
#pragma unroll
                for (int i = 0; i < d; ++i)
#pragma unroll
                    for (int j = 0; j < d; ++j) Pt[i * d + j] = Pb[j * d + i];
            }
            for (int32_t q = qptr[u]; q < qptr[u + 1]; ++q)
            {
                T Qb[d * d];
                load_block<d, T>(Qv + (int64_t)q * d * d, Qb);
                const int32_t sl = find_col(ccol, c0, c1, qcol[q]);
                if (sl >= 0) mat_mul_acc<d, T>(Pt, Qb, Ac + (int64_t)sl * d * d);
            }
        }
    }
}

/* res = r - A x, one block row per thread */
template <int d, typename T>
__global__ void k_amg_residual(int64_t n, const int32_t* __restrict__ bptr, const int32_t* __restrict__ bcol,
                               const T* __restrict__ A, const T* __restrict__ r, const T* __restrict__ x, T* __restrict__ res,
                               const DevScalars* ds)
{
    AMG_STOP;
    GRID_STRIDE(u, n)
    {
        T y[d];
        bsr_row_product4<d, T>(bptr, bcol, A, x, u, y);
#pragma unroll
        for (int i = 0; i < d; ++i) res[u * d + i] = r[u * d + i] - y[i];
    }
}

/* k_amg_residual on the sliced-ELL copy of the finest level's matrix (the
   problem's H) */
template <int d, typename T>
__global__ void k_amg_residual_sell(int64_t n, const int32_t* __restrict__ sptr, const int32_t* __restrict__ scol,
                                    const T* __restrict__ As, const T* __restrict__ r, const T* __restrict__ x,
                                    T* __restrict__ res, const DevScalars* ds)
{
    AMG_STOP;
    GRID_STRIDE(u, n)
    {
        T y[d];
        sell_row_product<d, T>(sptr, scol, As, x, u, y);
#pragma unroll
        for (int i = 0; i < d; ++i) res[u * d + i] = r[u * d + i] - y[i];
    }
}

/* r_c(I) = sum_u P(u, I)^T res(u), x_c(I) = S_c(I) r_c(I): RestrictLanes<d>
   lanes per coarse row (32 / L rows per warp at once), lane k of a row taking
   its k-th, (k+L)-th, ... (u, P(u, I)) pair, then a fixed xor-shuffle tree
   within the row's lanes (deterministic).  Coarse rows have 20-40 pairs on
   the 2D levels: a warp per row left its dependent gathers one row deep. */
template <int d> struct RestrictLanes { static constexpr int value = d == 3 ? 16 : 8; };

template <int d, typename T>
__global__ void k_amg_restrict(int64_t nc, const int32_t* __restrict__ tptr, const int32_t* __restrict__ tu,
                               const int32_t* __restrict__ tp, const T* __restrict__ Pv, const T* __restrict__ res,
                               const T* __restrict__ dl1c, T* __restrict__ rc, T* __restrict__ xc, const DevScalars* ds)
{
    AMG_STOP;
    constexpr int L = RestrictLanes<d>::value, RPW = 32 / L;
    const int lane = threadIdx.x % L, sub = (threadIdx.x & 31) / L;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp * RPW; base < nc; base += n_warps * RPW)
    {
        const int64_t I = base + sub;
        T acc[d];
#pragma unroll
        for (int i = 0; i < d; ++i) acc[i] = T(0);
        if (I < nc)
            for (int32_t t = tptr[I] + lane; t < tptr[I + 1]; t += L)
            {
                const int64_t u = tu[t];
                T Pb[d * d], rv[d];
                load_block<d, T>(Pv + (int64_t)tp[t] * d * d, Pb);
                load_vec<d, T>(res + u * d, rv);
#pragma unroll
                for (int j = 0; j < d; ++j)
#pragma unroll
                    for (int i = 0; i < d; ++i) acc[j] += Pb[i * d + j] * rv[i];
            }
#pragma unroll
        for (int off = L / 2; off > 0; off >>= 1)
#pragma unroll
            for (int i = 0; i < d; ++i) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], off, L);
        if (I < nc && lane == 0)
        {
            T z[d];
            apply_dinv<d, T>(dl1c, I, acc, z);
#pragma unroll
            for (int i = 0; i < d; ++i) { rc[I * d + i] = acc[i]; xc[I * d + i] = z[i]; }
        }
    }
}

/* x += P x_c + S (res - Q x_c) = R x_c + S res (R = P - S Q, k_amg_q); top
   level (rz != NULL): also the PCG's r.z reduction, beta = r.z / rz_old
   (first: 0) and the breakdown test */
template <int d, typename T>
__global__ void __launch_bounds__(RED_THREADS) k_amg_post(int64_t n, const int32_t* __restrict__ qptr,
                                                          const int32_t* __restrict__ qcol, const T* __restrict__ Rv,
                                                          const T* __restrict__ dl1, const T* __restrict__ xc,
                                                          const T* __restrict__ res, T* __restrict__ x, const T* __restrict__ r,
                                                          double* partials, unsigned* counter, DevScalars* ds, int first)
{
    AMG_STOP;
    T part = T(0);
    GRID_STRIDE(u, n)
    {
        T rx[d], rv[d], s[d], xv[d];
        bsr_row_product4<d, T>(qptr, qcol, Rv, xc, u, rx);
        load_vec<d, T>(res + u * d, rv);
        apply_dinv<d, T>(dl1, u, rv, s);
        load_vec<d, T>(x + u * d, xv);
#pragma unroll
        for (int i = 0; i < d; ++i)
        {
            const T xn = xv[i] + rx[i] + s[i];
            xv[i] = xn;
            if (r) part += r[u * d + i] * xn;
        }
        store_vec<d, T>(x + u * d, xv);
    }
    if (!r) return;
    double v[1] = {as_double(part)}, tot[1];
    if (!grid_sum<1>(v, partials, counter, tot)) return;
    if (threadIdx.x == 0)
    {
        if (!(tot[0] > 0.0) || !isfinite(tot[0])) { ds->breakdown = 1; ds->done = 1; return; }
        ds->beta = first ? 0.0 : tot[0] / ds->rz;
        ds->rz = tot[0];
    }
}

/* coarsest level: x (already S r) plus AMG_COARSE_SWEEPS - 1 further l1
   block-Jacobi sweeps x += S (r - A x), in one thread block (w: scratch).
   CoarseLanes<d> lanes share a block row (lane l takes its blocks l, l + L,
   ...; a fixed xor-shuffle tree sums them): a coarse row of a tetrahedral
   mesh has 30-40 3 x 3 blocks, whose dependent loads one thread per row
   walked in sequence (95 us per call on the 48^3 cube, 12 sweeps). */
template <int d> struct CoarseLanes { static constexpr int value = d == 3 ? 16 : 4; };

template <int d, typename T>
__global__ void __launch_bounds__(AMG_COARSE_THREADS) k_amg_coarse(int64_t n, const int32_t* __restrict__ bptr,
                                                                   const int32_t* __restrict__ bcol, const T* __restrict__ A,
                                                                   const T* __restrict__ dl1, const T* __restrict__ r,
                                                                   T* __restrict__ x, T* __restrict__ w, const DevScalars* ds)
{
    AMG_STOP;
    constexpr int L = CoarseLanes<d>::value, RPP = AMG_COARSE_THREADS / L;   // rows per pass
    const int lane = threadIdx.x % L, sub = threadIdx.x / L;
    T* a = x;
    T* b = w;
    for (int k = 1; k < AMG_COARSE_SWEEPS; ++k)
    {
        for (int64_t base = 0; base < n; base += RPP)
        {
            const int64_t u = base + sub;
            T y[d];
#pragma unroll
            for (int i = 0; i < d; ++i) y[i] = T(0);
            if (u < n)
                for (int32_t q = bptr[u] + lane; q < bptr[u + 1]; q += L)
                {
                    const int64_t v = bcol[q];
                    T B[d * d], av[d];
                    load_block<d, T>(A + (int64_t)q * d * d, B);
                    load_vec<d, T>(a + v * d, av);
#pragma unroll
                    for (int i = 0; i < d; ++i)
#pragma unroll
                        for (int j = 0; j < d; ++j) y[i] += B[i * d + j] * av[j];
                }
#pragma unroll
            for (int off = L / 2; off > 0; off >>= 1)
#pragma unroll
                for (int i = 0; i < d; ++i) y[i] += __shfl_xor_sync(0xffffffffu, y[i], off, L);
            if (u < n && lane == 0)
            {
                T e[d], sv[d];
#pragma unroll
                for (int i = 0; i < d; ++i) e[i] = r[u * d + i] - y[i];
                apply_dinv<d, T>(dl1, u, e, sv);
#pragma unroll
                for (int i = 0; i < d; ++i) b[u * d + i] = a[u * d + i] + sv[i];
            }
        }
        __syncthreads();
        T* t = a; a = b; b = t;
    }
    if (a != x)
    {
        for (int64_t i = threadIdx.x; i < n * d; i += blockDim.x) x[i] = a[i];
    }
}

/* CG restart under the V-cycle: z = S_0 r (pre-smoothing), p = Ap = 0 */
template <int d, typename T>
__global__ void k_amg_start(int64_t n, const T* __restrict__ r, const T* __restrict__ dl1, T* __restrict__ z, T* __restrict__ p,
                            T* __restrict__ Ap, const DevScalars* ds)
{
    AMG_STOP;
    GRID_STRIDE(u, n)
    {
        T rv[d], zv[d];
        load_vec<d, T>(r + u * d, rv);
        apply_dinv<d, T>(dl1, u, rv, zv);
#pragma unroll
        for (int i = 0; i < d; ++i) { z[u * d + i] = zv[i]; p[u * d + i] = T(0); Ap[u * d + i] = T(0); }
    }
}

/* after the SpMV: x += alpha p, r -= alpha Ap, r.r (the last block counts the
   iteration and sets the stop flag), z = S_0 r (the V-cycle's pre-smoothing) */
template <int d, typename T>
__global__ void __launch_bounds__(RED_THREADS) k_amg_update(int64_t n, T* __restrict__ x, T* __restrict__ r,
                                                            const T* __restrict__ p, const T* __restrict__ Ap,
                                                            const T* __restrict__ dl1, T* __restrict__ z, double* partials,
                                                            unsigned* counter, DevScalars* ds)
{
    AMG_STOP;
    const T alpha = from_double<T>(ds->alpha);
    T part = T(0);
    GRID_STRIDE(u, n)
    {
        T xv[d], pv[d], rv[d], av[d], zv[d];
        load_vec<d, T>(x + u * d, xv);
        load_vec<d, T>(p + u * d, pv);
        load_vec<d, T>(r + u * d, rv);
        load_vec<d, T>(Ap + u * d, av);
#pragma unroll
        for (int i = 0; i < d; ++i)
        {
            xv[i] += alpha * pv[i];
            rv[i] -= alpha * av[i];
            part += rv[i] * rv[i];
        }
        store_vec<d, T>(x + u * d, xv);
        store_vec<d, T>(r + u * d, rv);
        apply_dinv<d, T>(dl1, u, rv, zv);
        store_vec<d, T>(z + u * d, zv);
    }
    double v[1] = {as_double(part)}, tot[1];
    if (!grid_sum<1>(v, partials, counter, tot)) return;
    if (threadIdx.x == 0)
    {
        ds->rr = tot[0];
        ds->iters += 1;
        if (tot[0] <= ds->tol2 || ds->iters >= ds->max_iters || !isfinite(tot[0])) ds->done = 1;
    }
}

/* ---- host launchers ------------------------------------------------------------- */
/* a grid for n rows: enough blocks to cover them once, at most the reduction grid */
static unsigned grid_for(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(RED_BLOCKS, (n + RED_THREADS - 1) / RED_THREADS)); }

/* a grid of 256-thread blocks giving each of n rows its own group of
   32 / rows_per_warp lanes, at most 8 x RED_BLOCKS blocks (grid-stride beyond) */
static unsigned warp_grid(int64_t n, int rows_per_warp = 1)
{
    const int64_t warps = (n + rows_per_warp - 1) / rows_per_warp;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(8 * RED_BLOCKS, (warps + 7) / 8));
}

template <typename T>
static const T* level_A(const Problem& P, size_t l) { return l == 0 ? (const T*)P.H : (const T*)P.amg[l].A; }

/* the V-cycle below level l: on entry L.r holds the level's right-hand side
   (level 0: r) and x its pre-smoothed start S r; on exit x holds the result
   (the level-0 call reduces r.z into the PCG scalars) */
template <int d, typename T>
static void vcycle_from(Problem& P, size_t l, const T* r, T* x, int first)
{
    cudaStream_t s = P.stream;
    AmgLevel& L = P.amg[l];
    const T* A = level_A<T>(P, l);
    const DevScalars* ds = P.ds;
    if (l + 1 == P.amg.size())
    {
        k_amg_coarse<d, T><<<1, AMG_COARSE_THREADS, 0, s>>>(L.n, L.bptr, L.bcol, A, (const T*)L.dl1, r, x, (T*)L.w, ds);
        P.n_launches += 1;
        return;
    }
    AmgLevel& C = P.amg[l + 1];
    const unsigned g = grid_for(L.n);
    const SellView sv = l == 0 ? sell_view(P, A) : SellView{nullptr, nullptr, nullptr};
    if (sv.Hs)
        k_amg_residual_sell<d, T><<<g, RED_THREADS, 0, s>>>(L.n, sv.sptr, sv.scol, (const T*)sv.Hs, r, x, (T*)L.res, ds);
    else
        k_amg_residual<d, T><<<g, RED_THREADS, 0, s>>>(L.n, L.bptr, L.bcol, A, r, x, (T*)L.res, ds);
    k_amg_restrict<d, T><<<warp_grid(C.n, 32 / RestrictLanes<d>::value), RED_THREADS, 0, s>>>(C.n, L.tptr, L.tu, L.tp, (const T*)L.Pv, (const T*)L.res,
                                                                (const T*)C.dl1, (T*)C.r, (T*)C.x, ds);
    P.n_launches += 2;
    vcycle_from<d, T>(P, l + 1, (const T*)C.r, (T*)C.x, first);
    if (l == 0)
        k_amg_post<d, T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(L.n, L.qptr, L.qcol, (const T*)L.Rv, (const T*)L.dl1,
                                                            (const T*)C.x, (const T*)L.res, x, r, P.partials,
                                                            P.counters + 9, P.ds, first);
    else
        k_amg_post<d, T><<<g, RED_THREADS, 0, s>>>(L.n, L.qptr, L.qcol, (const T*)L.Rv, (const T*)L.dl1, (const T*)C.x,
                                                   (const T*)L.res, x, nullptr, nullptr, nullptr, P.ds, first);
    P.n_launches += 1;
}

template <int d, typename T>
static void apply(Problem& P, int mode, T* xs, T* r, T* z, T* p, T* Ap)
{
    cudaStream_t s = P.stream;
    AmgLevel& L = P.amg[0];
    if (mode == 0)
        k_amg_start<d, T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(L.n, r, (const T*)L.dl1, z, p, Ap, P.ds);
    else
        k_amg_update<d, T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(L.n, xs, r, p, Ap, (const T*)L.dl1, z, P.partials,
                                                              P.counters + 2, P.ds);
    P.n_launches += 1;
    vcycle_from<d, T>(P, 0, r, z, mode == 0);   // the solver uses hierarchies of two or more levels
}

template <int d, typename T>
static void values(Problem& P)
{
    cudaStream_t s = P.stream;
    for (size_t l = 0; l < P.amg.size(); ++l)
    {
        AmgLevel& L = P.amg[l];
        const T* A = level_A<T>(P, l);
        if (l > 0)
        {
            AmgLevel& F = P.amg[l - 1];
            if (L.max_row <= AMG_ROW_CAP)
            {
                const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>(8 * RED_BLOCKS, (L.n + AMG_SETUP_WARPS - 1) / AMG_SETUP_WARPS));
                k_amg_galerkin<d, T><<<g, AMG_SETUP_WARPS * 32, 0, s>>>(L.n, F.tptr, F.tu, F.tp, (const T*)F.Pv, F.qptr,
                                                                        F.qcol, (const T*)F.Qv, L.bptr, L.bcol, (T*)L.A);
            }
            else
                k_amg_galerkin_rows<d, T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(L.n, F.tptr, F.tu, F.tp, (const T*)F.Pv, F.qptr,
                                                                             F.qcol, (const T*)F.Qv, L.bptr, L.bcol, (T*)L.A);
            P.n_launches += 1;
        }
        k_amg_diag<d, T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(L.n, L.bptr, L.bcol, L.diag, A, (T*)L.dl1);
        P.n_launches += 1;
        if (l + 1 == P.amg.size()) break;
        k_amg_prolongator<d, T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(L.n, L.bptr, L.pslot, L.pptr, L.pcol, L.pdiag,
                                                                   L.cscale, A, (const T*)L.dl1, (T*)L.Pv);
        k_amg_q<d, T><<<(unsigned)std::min<int64_t>(8 * RED_BLOCKS, (L.nq + RED_THREADS - 1) / RED_THREADS + 1), RED_THREADS,
                        0, s>>>(L.nq, L.qlptr, L.qla, L.qlp, L.qrow, L.qpb, A, (const T*)L.Pv, (const T*)L.dl1, (T*)L.Qv,
                                (T*)L.Rv);
        P.n_launches += 2;
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
    P.amg_values_ready = true;
    return TAD_OK;
}

void amg_apply(Problem& P, int precision, int mode, void* xs, void* r, void* z, void* p, void* Ap)
{
    const bool f32 = precision == TAD_PREC_MIXED;
#define TAD_AMG_APPLY(D)                                                                                             \
    f32 ? apply<D, float>(P, mode, (float*)xs, (float*)r, (float*)z, (float*)p, (float*)Ap)                          \
        : apply<D, double>(P, mode, (double*)xs, (double*)r, (double*)z, (double*)p, (double*)Ap)
    switch (P.d)
    {
    case 1: TAD_AMG_APPLY(1); break;
    case 2: TAD_AMG_APPLY(2); break;
    default: TAD_AMG_APPLY(3); break;
    }
#undef TAD_AMG_APPLY
}

int amg_levels(const Problem& P) { return (int)P.amg.size(); }

} // namespace tadlib
