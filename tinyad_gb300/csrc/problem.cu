/*
 * Problem lifecycle, sparsity-pattern construction and the evaluation entry
 * points of the C ABI (include/tad.h).
 *
 * The reference re-derives the pattern on every eval_with_hessian_proj call:
 * it emits k^2 triplets per element and Eigen's setFromTriplets sorts and
 * sums them (include/TinyAD/Detail/ScalarFunctionImpl.hh:378-399).  Here the
 * pattern is built once on the host when the problem is finalised: a block
 * sparse row (BSR) structure with d x d blocks, and for every block the list
 * of element pair blocks that add into it, in element order -- the order in
 * which setFromTriplets sums duplicates.  Every later assembly is a
 * deterministic gather over those lists (kernels.cu), with no atomics and no
 * triplets.
 */
#include <algorithm>
#include <cstring>
#include <mutex>
#include <numeric>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "internal.hh"

namespace tadlib {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }

static tad_status fail(tad_status s, const std::string& msg)
{
    set_error(msg);
    return s;
}

static int builtin_dim_ok(int energy, int d, int N, int n_params)
{
    switch (energy)
    {
    case TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI: return d == 2 && N == 3 && n_params == 5;
    case TAD_ENERGY_SYMMETRIC_DIRICHLET_TET: return d == 3 && N == 4 && n_params == 10;
    case TAD_ENERGY_POSITION_PENALTY: return N == 1 && d >= 1 && d <= 3 && n_params == d + 1;
    case TAD_ENERGY_QUADRATIC:
    {
        const int k = d * N;
        const bool shape = (N == 1 && d >= 1 && d <= 3) || (N == 2 && d <= 2);
        return shape && n_params == k * k + k + 1;
    }
    case TAD_ENERGY_DIRICHLET_TRI: return N == 3 && (d == 1 || d == 2 || d == 3) && n_params == 1;
    }
    return 0;
}

tad_status launch_builtin(Problem& P, Term& T, const tad_term_eval_args& a)
{
    if (T.M > 0) return launch_builtin_vec(P, T, a);
    switch (T.energy)
    {
    case TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI:
    case TAD_ENERGY_DIRICHLET_TRI:
        return launch_builtin_tri(P, T, a);
    case TAD_ENERGY_SYMMETRIC_DIRICHLET_TET:
        return launch_builtin_tet(P, T, a);
    default:
        return launch_builtin_misc(P, T, a);
    }
}

template <typename X>
static cudaError_t dalloc(X** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void**)p, count * sizeof(X));
}

static void dfree(void* p)
{
    if (p) cudaFree(p);
}

tad_status check_device_error(Problem& P)
{
    TAD_CUDA_TRY(cudaMemcpyAsync(P.err_h, P.err, sizeof(int32_t), cudaMemcpyDeviceToHost, P.stream));
    TAD_CUDA_TRY(cudaStreamSynchronize(P.stream));
    const int32_t e = *P.err_h;
    if (e == 0) return TAD_OK;
    TAD_CUDA_TRY(cudaMemsetAsync(P.err, 0, sizeof(int32_t), P.stream));
    if (e & 2) return fail(TAD_ERR_TOO_MANY_VARS, "Too many variables requested via element.variables(...).");
    if (e & 1) return fail(TAD_ERR_ARG, "element accessed a variable handle outside its recorded access list");
    if (e & 4) return fail(TAD_ERR_NONFINITE, "Assertion failed: Not finite (element gradient or Hessian)");
    if (e & 8) return fail(TAD_ERR_TIMEOUT, "a bounded device-side wait gave up");
    if (e & 16) return fail(TAD_ERR_ARG, "HESSIAN_PROJ element kernel launched without tad_term_eval_args.proj_list_d");
    return fail(TAD_ERR_CUDA, "device error word " + std::to_string(e));
}

/* ------------------------------------------------------------------------ */
/* pattern construction                                                      */
/* ------------------------------------------------------------------------ */
static tad_status build_pattern(Problem& P)
{
    const int64_t nh = P.n_handles;
    const int nterm = (int)P.terms.size();
    // handle -> element slots (global slot ids), in (term, element, slot) order
    std::vector<int64_t> cnt(nh + 1, 0);
    for (const Term& T : P.terms)
        for (int64_t i = 0; i < T.n_elem * T.N; ++i)
            if (T.rec_h[i] >= 0) cnt[T.rec_h[i] + 1]++;
    for (int64_t v = 0; v < nh; ++v) cnt[v + 1] += cnt[v];
    const int64_t ninc = cnt[nh];
    if (P.n_slots_total >= (int64_t(1) << 31) || P.n_pairs_total >= (int64_t(1) << 31))
        return fail(TAD_ERR_ARG, "problem too large for 31-bit element block ids");
    std::vector<int32_t> gptr(nh + 1), gidx(std::max<int64_t>(ninc, 1));
    for (int64_t v = 0; v <= nh; ++v) gptr[v] = (int32_t)cnt[v];
    {
        std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
        for (const Term& T : P.terms)
            for (int64_t i = 0; i < T.n_elem * T.N; ++i)
                if (T.rec_h[i] >= 0) gidx[pos[T.rec_h[i]]++] = (int32_t)(T.slot_off + i);
    }
    std::vector<int64_t> slot_off(nterm);
    for (int t = 0; t < nterm; ++t) slot_off[t] = P.terms[t].slot_off;
    auto decode = [&](int32_t s, int& t, int64_t& e, int& a) {
        t = (int)(std::upper_bound(slot_off.begin(), slot_off.end(), (int64_t)s) - slot_off.begin()) - 1;
        const int64_t loc = s - slot_off[t];
        e = loc / P.terms[t].N;
        a = (int)(loc % P.terms[t].N);
    };
    // block rows
    std::vector<std::vector<int32_t>> rows(nh);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t u = 0; u < nh; ++u)
    {
        std::vector<int32_t>& c = rows[u];
        for (int32_t q = gptr[u]; q < gptr[u + 1]; ++q)
        {
            int t; int64_t e; int a;
            decode(gidx[q], t, e, a);
            const Term& T = P.terms[t];
            for (int b = 0; b < T.N; ++b)
            {
                const int32_t w = T.rec_h[e * T.N + b];
                if (w >= 0) c.push_back(w);
            }
        }
        std::sort(c.begin(), c.end());
        c.erase(std::unique(c.begin(), c.end()), c.end());
    }
    std::vector<int32_t> bptr(nh + 1, 0);
    for (int64_t u = 0; u < nh; ++u) bptr[u + 1] = bptr[u] + (int32_t)rows[u].size();
    const int64_t nb = bptr[nh];
    std::vector<int32_t> bcol(std::max<int64_t>(nb, 1)), diag(std::max<int64_t>(nh, 1), -1);
    // contributions: count per block, then fill in element order
    std::vector<int32_t> ccnt(nb + 1, 0);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t u = 0; u < nh; ++u)
    {
        const std::vector<int32_t>& c = rows[u];
        std::copy(c.begin(), c.end(), bcol.begin() + bptr[u]);
        auto it = std::lower_bound(c.begin(), c.end(), (int32_t)u);
        if (it != c.end() && *it == u) diag[u] = bptr[u] + (int32_t)(it - c.begin());
        for (int32_t q = gptr[u]; q < gptr[u + 1]; ++q)
        {
            int t; int64_t e; int a;
            decode(gidx[q], t, e, a);
            const Term& T = P.terms[t];
            for (int b = 0; b < T.N; ++b)
            {
                const int32_t w = T.rec_h[e * T.N + b];
                if (w < 0) continue;
                const int64_t j = std::lower_bound(c.begin(), c.end(), w) - c.begin();
                ccnt[bptr[u] + j + 1]++;
            }
        }
    }
    for (int64_t b = 0; b < nb; ++b) ccnt[b + 1] += ccnt[b];
    const int64_t ncontrib = ccnt[nb];
    std::vector<int32_t> cidx(std::max<int64_t>(ncontrib, 1));
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t u = 0; u < nh; ++u)
    {
        const std::vector<int32_t>& c = rows[u];
        std::vector<int32_t> fillpos(c.size());
        for (size_t j = 0; j < c.size(); ++j) fillpos[j] = ccnt[bptr[u] + j];
        for (int32_t q = gptr[u]; q < gptr[u + 1]; ++q)
        {
            int t; int64_t e; int a;
            decode(gidx[q], t, e, a);
            const Term& T = P.terms[t];
            const int NP = T.N * (T.N + 1) / 2;
            for (int b = 0; b < T.N; ++b)
            {
                const int32_t w = T.rec_h[e * T.N + b];
                if (w < 0) continue;
                const int64_t j = std::lower_bound(c.begin(), c.end(), w) - c.begin();
                const int lo = std::min(a, b), hi = std::max(a, b);
                const int pidx = lo * T.N - (lo * (lo - 1)) / 2 + (hi - lo);
                const int64_t id = T.pair_off + e * NP + pidx;
                cidx[fillpos[j]++] = (int32_t)id | (a > b ? (int32_t)0x80000000 : 0);
            }
        }
    }
    P.nb = nb;
    P.ncontrib = ncontrib;
    P.ninc = ninc;
    P.bptr_h = bptr;
    P.bcol_h.assign(bcol.begin(), bcol.begin() + nb);
    TAD_CUDA_TRY(dalloc(&P.bptr, nh + 1));
    TAD_CUDA_TRY(dalloc(&P.bcol, nb));
    TAD_CUDA_TRY(dalloc(&P.diag, nh));
    TAD_CUDA_TRY(dalloc(&P.cptr, nb + 1));
    TAD_CUDA_TRY(dalloc(&P.cidx, ncontrib));
    TAD_CUDA_TRY(dalloc(&P.gptr, nh + 1));
    TAD_CUDA_TRY(dalloc(&P.gidx, ninc));
    TAD_CUDA_TRY(cudaMemcpy(P.bptr, bptr.data(), (nh + 1) * 4, cudaMemcpyHostToDevice));
    TAD_CUDA_TRY(cudaMemcpy(P.bcol, bcol.data(), nb * 4, cudaMemcpyHostToDevice));
    TAD_CUDA_TRY(cudaMemcpy(P.diag, diag.data(), nh * 4, cudaMemcpyHostToDevice));
    TAD_CUDA_TRY(cudaMemcpy(P.cptr, ccnt.data(), (nb + 1) * 4, cudaMemcpyHostToDevice));
    TAD_CUDA_TRY(cudaMemcpy(P.cidx, cidx.data(), ncontrib * 4, cudaMemcpyHostToDevice));
    TAD_CUDA_TRY(cudaMemcpy(P.gptr, gptr.data(), (nh + 1) * 4, cudaMemcpyHostToDevice));
    TAD_CUDA_TRY(cudaMemcpy(P.gidx, gidx.data(), ninc * 4, cudaMemcpyHostToDevice));
    return TAD_OK;
}

/* The sliced-ELL layout of H's pattern (Problem::sptr/scol/spos/sdiag) and
   the zeroed copy Hs, for 3 x 3 blocks.  Measured per PCG SpMV (ncu, cold
   cache): 663,552 tets (3 x 3 blocks, ~15 per row) 30.9 us for the BSR form
   with 8 lanes per row, 22.0 us on the copy; the 1.64M-face disk (2 x 2
   blocks, ~7 per row, each warp's rows already one contiguous 3.6 KB range)
   31.2 us against 31.8 us, while the second write made its assembly 18 us
   slower -- so 2 x 2 problems keep the BSR form only.  Left out too when the
   padding would add more than half the blocks of the pattern. */
static tad_status build_sell(Problem& P)
{
    if (P.d != 3) return TAD_OK;
    const int64_t nh = P.n_handles, ns = (nh + 31) / 32;
    std::vector<int32_t> sptr(ns + 1, 0);
    for (int64_t sl = 0; sl < ns; ++sl)
    {
        int32_t mx = 0;
        for (int64_t u = sl * 32; u < std::min<int64_t>(nh, sl * 32 + 32); ++u) mx = std::max(mx, P.bptr_h[u + 1] - P.bptr_h[u]);
        if ((int64_t)sptr[sl] + 32 * (int64_t)mx >= INT32_MAX) return TAD_OK;
        sptr[sl + 1] = sptr[sl] + 32 * mx;
    }
    const int64_t slots = sptr[ns];
    if (slots > P.nb + P.nb / 2) return TAD_OK;
    std::vector<int32_t> scol(slots), spos(P.nb), sdiag(nh, -1);
    for (int64_t sl = 0; sl < ns; ++sl)
        for (int lane = 0; lane < 32; ++lane)
        {
            const int64_t u = sl * 32 + lane;
            const int32_t len = u < nh ? P.bptr_h[u + 1] - P.bptr_h[u] : 0;
            for (int32_t j = 0; (int64_t)sptr[sl] + 32 * j < sptr[sl + 1]; ++j)
            {
                const int64_t q = sptr[sl] + 32 * (int64_t)j + lane;
                if (j < len)
                {
                    const int32_t b = P.bptr_h[u] + j;
                    scol[q] = P.bcol_h[b];
                    spos[b] = (int32_t)q;
                    if (P.bcol_h[b] == u) sdiag[u] = (int32_t)q;
                }
                else scol[q] = (int32_t)std::min<int64_t>(u, nh - 1);   // a zero block; any valid column
            }
        }
    P.n_slots = slots;
    TAD_CUDA_TRY(dalloc(&P.sptr, ns + 1));
    TAD_CUDA_TRY(dalloc(&P.scol, slots));
    TAD_CUDA_TRY(dalloc(&P.spos, P.nb));
    TAD_CUDA_TRY(dalloc(&P.sdiag, nh));
    TAD_CUDA_TRY(dalloc((double**)&P.Hs, slots * P.d * P.d));
    TAD_CUDA_TRY(cudaMemcpy(P.sptr, sptr.data(), (ns + 1) * 4, cudaMemcpyHostToDevice));
    TAD_CUDA_TRY(cudaMemcpy(P.scol, scol.data(), slots * 4, cudaMemcpyHostToDevice));
    TAD_CUDA_TRY(cudaMemcpy(P.spos, spos.data(), P.nb * 4, cudaMemcpyHostToDevice));
    TAD_CUDA_TRY(cudaMemcpy(P.sdiag, sdiag.data(), nh * 4, cudaMemcpyHostToDevice));
    TAD_CUDA_TRY(cudaMemset(P.Hs, 0, slots * P.d * P.d * sizeof(double)));
    P.Hs_of = P.H;
    return TAD_OK;
}

tad_status ensure_finalized(Problem& P)
{
    if (P.finalized) return TAD_OK;
    if (P.terms.empty()) return fail(TAD_ERR_STATE, "problem has no elements");
    // offsets
    int64_t eo = 0, so = 0, po = 0, oo = 0, jo = 0, ho = 0;
    for (Term& T : P.terms)
    {
        T.elem_off = eo; T.slot_off = so; T.pair_off = po;
        eo += T.n_elem; so += T.n_elem * T.N; po += T.n_elem * (T.N * (T.N + 1) / 2);
        const int64_t k = (int64_t)P.d * T.N;
        T.out_off = oo; T.jac_off = jo; T.hv_off = ho;
        oo += T.n_elem * T.M; jo += T.n_elem * T.M * k; ho += T.n_elem * T.M * (k * (k + 1) / 2);
    }
    P.n_elem_total = eo; P.n_slots_total = so; P.n_pairs_total = po;
    P.n_outputs_total = oo; P.jac_size = jo; P.hv_size = ho;
    dfree(P.ef); dfree(P.eg); dfree(P.eH);
    TAD_CUDA_TRY(dalloc(&P.ef, (size_t)eo * LS_BATCH));
    TAD_CUDA_TRY(dalloc(&P.eg, (size_t)so * P.d));
    P.eH_bytes = (size_t)po * P.d * P.d * sizeof(double);
    TAD_CUDA_TRY(cudaMalloc(&P.eH, std::max<size_t>(P.eH_bytes, 8)));
    {
        int64_t mx = 0;
        for (const Term& T : P.terms) mx = std::max(mx, T.n_elem);
        if (mx >= (int64_t)UINT32_MAX) return fail(TAD_ERR_ARG, "a term has 2^32 - 1 or more elements");
        dfree(P.proj_list);
        TAD_CUDA_TRY(cudaMalloc(&P.proj_list, (size_t)(mx + 1) * sizeof(uint32_t)));
        TAD_CUDA_TRY(cudaMemsetAsync(P.proj_list, 0, sizeof(uint32_t), P.stream));
    }
    // record access order of custom terms (x = 0)
    for (Term& T : P.terms)
    {
        if (T.energy >= 0) continue;
        TAD_CUDA_TRY(cudaMemsetAsync(P.x, 0, P.n_vars * sizeof(double), P.stream));
        TAD_CUDA_TRY(dalloc(&T.rec_d, T.n_elem * T.N));
        tad_term_eval_args a{};
        a.mode = TAD_MODE_RECORD;
        a.n_elem = T.n_elem; a.valence = T.N; a.var_dim = P.d; a.n_outputs = T.M;
        a.x_d = P.x; a.record_d = T.rec_d; a.error_d = P.err; a.stream = P.stream;
        const int rc = T.fn(T.user, &a);
        if (rc != 0) return fail(TAD_ERR_ARG, "custom term callback failed while recording");
        tad_status s = check_device_error(P);
        if (s != TAD_OK) return s;
        T.rec_h.resize(T.n_elem * T.N);
        TAD_CUDA_TRY(cudaMemcpy(T.rec_h.data(), T.rec_d, T.n_elem * T.N * 4, cudaMemcpyDeviceToHost));
        for (int32_t v : T.rec_h)
            if (v >= P.n_handles) return fail(TAD_ERR_ARG, "element accessed a handle out of range");
    }
    tad_status s = build_pattern(P);
    if (s != TAD_OK) return s;
    const int64_t n = P.n_vars, nh = P.n_handles, dd = P.d * P.d;
    TAD_CUDA_TRY(dalloc((double**)&P.H, P.nb * dd));
    s = build_sell(P);
    if (s != TAD_OK) return s;
    TAD_CUDA_TRY(dalloc(&P.csr_tmp, P.nb * dd));
    TAD_CUDA_TRY(dalloc(&P.r, n)); TAD_CUDA_TRY(dalloc(&P.z, n)); TAD_CUDA_TRY(dalloc(&P.p, n));
    TAD_CUDA_TRY(dalloc(&P.Ap, n)); TAD_CUDA_TRY(dalloc(&P.dx, n)); TAD_CUDA_TRY(dalloc(&P.dinv, nh * dd));
    TAD_CUDA_TRY(dalloc(&P.rhs, n)); TAD_CUDA_TRY(dalloc(&P.res, n));
    TAD_CUDA_TRY(dalloc(&P.r32, n)); TAD_CUDA_TRY(dalloc(&P.z32, n)); TAD_CUDA_TRY(dalloc(&P.p32, n));
    TAD_CUDA_TRY(dalloc(&P.Ap32, n)); TAD_CUDA_TRY(dalloc(&P.dx32, n)); TAD_CUDA_TRY(dalloc(&P.dinv32, nh * dd));
    P.finalized = true;
    // the AMG hierarchy's patterns (host work, once per problem) here rather
    // than inside the first solve that needs them
    if (P.settings.preconditioner == 1)
    {
        s = amg_build(P);
        if (s != TAD_OK) return s;
    }
    // and the Newton loop's captured PCG iteration graphs
    return prepare_solver_graphs(P);
}

/* ------------------------------------------------------------------------ */
/* evaluation                                                                */
/* ------------------------------------------------------------------------ */
tad_status eval_elements(Problem& P, int mode, const double* x, double eps, int precision,
                         const double* dir, int n_steps)
{
    P.spec_valid = false;   // the element and assembled buffers are about to change
    for (Term& T : P.terms)
    {
        tad_term_eval_args a{};
        a.mode = mode;
        a.precision = precision;
        a.n_elem = T.n_elem; a.valence = T.N; a.var_dim = P.d;
        a.x_d = x; a.dir_d = dir; a.steps_d = P.steps; a.n_steps = n_steps;
        a.proj_eps = eps;
        a.handles_d = T.rec_d;
        a.out_f_d = P.ef + T.elem_off;
        a.out_g_d = P.eg + T.slot_off * P.d;
        a.out_H_d = (char*)P.eH + T.pair_off * P.d * P.d * (precision == TAD_PREC_MIXED ? sizeof(float) : sizeof(double));
        a.error_d = P.err;
        a.stream = P.stream;
        a.proj_list_d = P.proj_list;
        a.active_d = P.launch_guard;
        a.n_outputs = T.M;
        if (T.M > 0)
        {
            a.out_r_d = (P.vec_outputs >= 1 && P.vr) ? P.vr + T.out_off : nullptr;
            a.out_J_d = (P.vec_outputs >= 2 && P.vJ) ? P.vJ + T.jac_off : nullptr;
            a.out_Hv_d = (P.vec_outputs >= 3 && P.vHv) ? P.vHv + T.hv_off : nullptr;
        }
        if (mode == TAD_MODE_LINESEARCH) a.f_row_stride = P.n_elem_total;
        tad_status s = T.energy >= 0 ? launch_builtin(P, T, a)
                                     : (T.fn(T.user, &a) == 0 ? TAD_OK : fail(TAD_ERR_ARG, "custom term failed"));
        if (s != TAD_OK) return s;
        if (T.n_elem > 0) P.n_launches += 1;
    }
    TAD_CUDA_TRY(cudaGetLastError());
    return TAD_OK;
}

tad_status assemble(Problem& P, bool gradient, bool hessian, int precision, double* f_dst, bool newton_rhs)
{
    launch_reduce_f(P, 1, f_dst ? f_dst : &P.ds->f);
    // the mixed second-order element kernels write double-float gradient pairs
    const bool pairs = precision == TAD_PREC_MIXED && hessian;
    if (gradient && newton_rhs) launch_assemble_grad_newton(P, precision, pairs);
    else if (gradient) launch_assemble_grad(P, precision, pairs);
    if (hessian) launch_assemble_hess(P, precision);
    P.n_launches += 1 + (gradient ? 1 : 0) + (hessian ? 1 : 0);
    TAD_CUDA_TRY(cudaGetLastError());
    return TAD_OK;
}

tad_status eval_full(Problem& P, const double* x, int mode, double eps, int precision)
{
    tad_status s = ensure_finalized(P);
    if (s != TAD_OK) return s;
    s = eval_elements(P, mode, x, eps, precision);
    if (s != TAD_OK) return s;
    return assemble(P, mode >= TAD_MODE_GRADIENT, mode >= TAD_MODE_HESSIAN, precision);
}

} // namespace tadlib

using namespace tadlib;

/* ------------------------------------------------------------------------ */
/* C ABI                                                                     */
/* ------------------------------------------------------------------------ */

extern "C" {

TAD_API void tad_settings_default(tad_settings* s)
{
    if (!s) return;
    s->precision = TAD_PREC_FP64;
    s->pcg_max_iters = 1000;
    s->pcg_rel_tol = 1e-10;
    s->refine_max_iters = 4;
    s->refine_rel_tol = 1e-10;
    s->ls_max_iters = 64;
    s->ls_shrink = 0.8;
    s->ls_armijo = 1e-4;
    s->forcing = 0;
    s->verbose = 0;
    s->preconditioner = 1;
}

TAD_API const char* tad_last_error_message(void) { return g_last_error.c_str(); }
TAD_API const char* tad_version(void) { return "tad-gb300 0.1 (sm_103a)"; }

TAD_API tad_status tad_problem_create(int var_dim, int64_t n_handles, const tad_settings* settings, tad_problem** out)
{
    if (!out) return fail(TAD_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (var_dim < 1 || var_dim > 3) return fail(TAD_ERR_ARG, "Variable dimension needs to be 1, 2 or 3.");
    if (n_handles <= 0) return fail(TAD_ERR_ARG, "Assertion failed: !variable_handles.empty()");
    if ((int64_t)var_dim * n_handles >= (int64_t(1) << 31)) return fail(TAD_ERR_ARG, "too many variables");
    tad_problem* P = new tad_problem();
    P->d = var_dim;
    P->n_handles = n_handles;
    P->n_vars = var_dim * n_handles;
    if (settings) P->settings = *settings;
    else tad_settings_default(&P->settings);
    P->precision = P->settings.precision;
    TAD_CUDA_TRY(cudaGetDevice(&P->device));
    TAD_CUDA_TRY(cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking));
    TAD_CUDA_TRY(cudaStreamCreateWithFlags(&P->stream2, cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&P->ev_in, &P->ev_xt, &P->ev_out}) TAD_CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    TAD_CUDA_TRY(cudaMalloc(&P->ds, sizeof(DevScalars)));
    TAD_CUDA_TRY(cudaMemset(P->ds, 0, sizeof(DevScalars)));
    TAD_CUDA_TRY(cudaMallocHost(&P->hs, sizeof(DevScalars)));
    TAD_CUDA_TRY(cudaMalloc(&P->err, sizeof(int32_t)));
    TAD_CUDA_TRY(cudaMemset(P->err, 0, sizeof(int32_t)));
    TAD_CUDA_TRY(cudaMallocHost(&P->err_h, sizeof(int32_t)));
    TAD_CUDA_TRY(cudaMalloc(&P->counters, 64 * sizeof(unsigned)));
    TAD_CUDA_TRY(cudaMemset(P->counters, 0, 64 * sizeof(unsigned)));
    static_assert(PCG_BLOCKS * 3 <= RED_BLOCKS * LS_BATCH * 4, "PCG grid sums must fit the partials buffer");
    TAD_CUDA_TRY(cudaMalloc(&P->partials, (size_t)RED_BLOCKS * LS_BATCH * 4 * sizeof(double)));
    TAD_CUDA_TRY(cudaMalloc(&P->steps, 64 * sizeof(double)));
    TAD_CUDA_TRY(cudaMalloc(&P->x, P->n_vars * sizeof(double)));
    TAD_CUDA_TRY(cudaMemset(P->x, 0, P->n_vars * sizeof(double)));
    TAD_CUDA_TRY(cudaMalloc(&P->g, P->n_vars * sizeof(double)));
    for (auto& e : P->ev) TAD_CUDA_TRY(cudaEventCreate(&e));
    *out = P;
    return TAD_OK;
}

TAD_API tad_status tad_problem_destroy(tad_problem* P)
{
    if (!P) return TAD_OK;
    cudaStreamSynchronize(P->stream);
    for (Term& T : P->terms) { dfree(T.vtx_d); dfree(T.prm_d); dfree(T.rec_d); }
    void* bufs[] = {P->ef, P->eg, P->eH, P->bptr, P->bcol, P->diag, P->cptr, P->cidx, P->gptr, P->gidx,
                    P->x, P->g, P->H, P->H64, P->csr_tmp, P->r, P->z, P->p, P->Ap, P->dx, P->dinv,
                    P->r32, P->z32, P->p32, P->Ap32, P->dx32, P->dinv32, P->rhs, P->res, P->steps,
                    P->partials, P->counters, P->ds, P->err, P->proj_list, P->steps_seq, P->x_trial,
                    P->last_x, P->diff_flag, P->sptr, P->scol, P->spos, P->sdiag, P->Hs};
    for (void* b : bufs) dfree(b);
    if (P->hs) cudaFreeHost(P->hs);
    if (P->err_h) cudaFreeHost(P->err_h);
    if (P->diff_flag_h) cudaFreeHost(P->diff_flag_h);
    if (P->pcg_graph) cudaGraphExecDestroy(P->pcg_graph);
    if (P->amg_graph) cudaGraphExecDestroy(P->amg_graph);
    if (P->Hd) cudaFree(P->Hd);
    if (P->corr) cudaFree(P->corr);
    amg_free(*P);
    for (auto& e : P->ev) if (e) cudaEventDestroy(e);
    for (auto& e : P->stage_ev) if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {P->ev_in, P->ev_xt, P->ev_out}) if (e) cudaEventDestroy(e);
    if (P->stream2) { cudaStreamSynchronize(P->stream2); cudaStreamDestroy(P->stream2); }
    if (P->stream) cudaStreamDestroy(P->stream);
    delete P;
    return TAD_OK;
}

TAD_API tad_status tad_problem_set_settings(tad_problem* P, const tad_settings* s)
{
    if (!P || !s) return fail(TAD_ERR_ARG, "NULL argument");
    P->settings = *s;
    P->precision = s->precision;
    P->g0_norm = 0.0;
    P->spec_valid = false;
    P->last_x_valid = false;
    return TAD_OK;
}

TAD_API int64_t tad_n_vars(const tad_problem* P) { return P ? P->n_vars : 0; }

/* a built-in term: element handles (deduplicated per element into the
   recorded first-access order) and parameters uploaded once */
static tad_status add_builtin_term(tad_problem* P, int energy, int valence, int n_outputs, int64_t n_elem,
                                   const int32_t* handles_h, const double* params_h, int n_params)
{
    Term T;
    T.energy = energy; T.N = valence; T.M = n_outputs; T.n_elem = n_elem; T.n_params = n_params;
    T.vtx_h.assign(handles_h, handles_h + n_elem * valence);
    T.rec_h.resize(n_elem * valence);
    for (int64_t e = 0; e < n_elem; ++e)
    {
        int n = 0;
        for (int a = 0; a < valence; ++a)
        {
            const int32_t v = T.vtx_h[e * valence + a];
            if (v < 0 || v >= P->n_handles)
                return fail(TAD_ERR_ARG, "Assertion failed: variable handle index out of range");
            bool seen = false;
            for (int b = 0; b < n; ++b) seen = seen || T.rec_h[e * valence + b] == v;
            if (!seen) T.rec_h[e * valence + n++] = v;
        }
        for (int a = n; a < valence; ++a) T.rec_h[e * valence + a] = -1;
    }
    TAD_CUDA_TRY(dalloc(&T.vtx_d, n_elem * valence));
    TAD_CUDA_TRY(dalloc(&T.rec_d, n_elem * valence));
    TAD_CUDA_TRY(dalloc(&T.prm_d, n_elem * n_params));
    TAD_CUDA_TRY(cudaMemcpy(T.vtx_d, T.vtx_h.data(), n_elem * valence * 4, cudaMemcpyHostToDevice));
    TAD_CUDA_TRY(cudaMemcpy(T.rec_d, T.rec_h.data(), n_elem * valence * 4, cudaMemcpyHostToDevice));
    if (n_elem * n_params > 0)
        TAD_CUDA_TRY(cudaMemcpy(T.prm_d, params_h, n_elem * n_params * sizeof(double), cudaMemcpyHostToDevice));
    P->terms.push_back(std::move(T));
    return TAD_OK;
}

TAD_API tad_status tad_add_elements(tad_problem* P, int energy, int valence, int64_t n_elem,
                                    const int32_t* handles_h, const double* params_h, int n_params)
{
    if (!P) return fail(TAD_ERR_ARG, "NULL problem");
    if (energy < 0 || energy >= TAD_ENERGY_COUNT_) return fail(TAD_ERR_ARG, "unknown energy");
    if (valence < 1 || valence > 4) return fail(TAD_ERR_ARG, "valence must be 1..4");
    if (n_elem < 0 || (n_elem > 0 && !handles_h)) return fail(TAD_ERR_ARG, "bad element array");
    if (!builtin_dim_ok(energy, P->d, valence, n_params))
        return fail(TAD_ERR_ARG, "energy not available for this (var_dim, valence, n_params)");
    if (P->finalized) return fail(TAD_ERR_STATE, "elements must be added before the first evaluation");
    if (P->kind == 2) return fail(TAD_ERR_STATE, "a problem holds either scalar or vector terms");
    P->kind = 1;
    return add_builtin_term(P, energy, valence, 0, n_elem, handles_h, params_h, n_params);
}

TAD_API tad_status tad_add_vector_elements(tad_problem* P, int energy, int valence, int n_outputs, int64_t n_elem,
                                           const int32_t* handles_h, const double* params_h, int n_params)
{
    if (!P) return fail(TAD_ERR_ARG, "NULL problem");
    if (n_elem < 0 || (n_elem > 0 && !handles_h)) return fail(TAD_ERR_ARG, "bad element array");
    const bool ok = (energy == TAD_VEC_SYMMETRIC_DIRICHLET_TRI && P->d == 2 && valence == 3 && n_outputs == 8 && n_params == 5) ||
                    (energy == TAD_VEC_POSITION && P->d >= 1 && P->d <= 3 && valence == 1 && n_outputs == P->d &&
                     n_params == P->d + 1);
    if (!ok) return fail(TAD_ERR_ARG, "vector energy not available for this (var_dim, valence, outputs, n_params)");
    if (P->finalized) return fail(TAD_ERR_STATE, "elements must be added before the first evaluation");
    if (P->kind == 1) return fail(TAD_ERR_STATE, "a problem holds either scalar or vector terms");
    P->kind = 2;
    return add_builtin_term(P, energy, valence, n_outputs, n_elem, handles_h, params_h, n_params);
}

TAD_API tad_status tad_add_elements_custom(tad_problem* P, int valence, int64_t n_elem, tad_term_eval_fn fn, void* user)
{
    if (!P || !fn) return fail(TAD_ERR_ARG, "NULL argument");
    if (valence < 1 || valence > 64) return fail(TAD_ERR_ARG, "valence must be 1..64");
    if (P->finalized) return fail(TAD_ERR_STATE, "elements must be added before the first evaluation");
    if (P->kind == 2) return fail(TAD_ERR_STATE, "a problem holds either scalar or vector terms");
    P->kind = 1;
    Term T;
    T.energy = -1; T.N = valence; T.n_elem = n_elem; T.fn = fn; T.user = user;
    P->terms.push_back(std::move(T));
    return TAD_OK;
}

TAD_API tad_status tad_add_vector_elements_custom(tad_problem* P, int valence, int n_outputs, int64_t n_elem,
                                                  tad_term_eval_fn fn, void* user)
{
    if (!P || !fn) return fail(TAD_ERR_ARG, "NULL argument");
    if (valence < 1 || valence > 64) return fail(TAD_ERR_ARG, "valence must be 1..64");
    if (n_outputs < 1) return fail(TAD_ERR_ARG, "outputs per element must be positive");
    if (n_elem < 0) return fail(TAD_ERR_ARG, "bad element count");
    if (P->finalized) return fail(TAD_ERR_STATE, "elements must be added before the first evaluation");
    if (P->kind == 1) return fail(TAD_ERR_STATE, "a problem holds either scalar or vector terms");
    P->kind = 2;
    Term T;
    T.energy = -1; T.N = valence; T.M = n_outputs; T.n_elem = n_elem; T.fn = fn; T.user = user;
    P->terms.push_back(std::move(T));
    return TAD_OK;
}

TAD_API tad_status tad_finalize(tad_problem* P)
{
    if (!P) return fail(TAD_ERR_ARG, "NULL problem");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    return ensure_finalized(*P);
}

TAD_API tad_status tad_hessian_nnz(tad_problem* P, int64_t* nnz)
{
    if (!P || !nnz) return fail(TAD_ERR_ARG, "NULL argument");
    tad_status s = ensure_finalized(*P);
    if (s != TAD_OK) return s;
    *nnz = P->nb * P->d * P->d;
    return TAD_OK;
}

TAD_API tad_status tad_hessian_pattern(tad_problem* P, int32_t* outer, int32_t* inner)
{
    if (!P || !outer || !inner) return fail(TAD_ERR_ARG, "NULL argument");
    tad_status s = ensure_finalized(*P);
    if (s != TAD_OK) return s;
    const int d = P->d;
    int64_t pos = 0;
    for (int64_t u = 0; u < P->n_handles; ++u)
        for (int p = 0; p < d; ++p)
        {
            outer[u * d + p] = (int32_t)pos;
            for (int32_t b = P->bptr_h[u]; b < P->bptr_h[u + 1]; ++b)
                for (int q = 0; q < d; ++q) inner[pos++] = P->bcol_h[b] * d + q;
        }
    outer[P->n_vars] = (int32_t)pos;
    return TAD_OK;
}

static tad_status eval_host(tad_problem* P, const double* x_h, int mode, double eps, double* f, double* g_h,
                            double* H_h, bool x_on_device)
{
    if (!P || !f) return fail(TAD_ERR_ARG, "NULL argument");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    tad_status s = ensure_finalized(*P);
    if (s != TAD_OK) return s;
    if (x_on_device) TAD_CUDA_TRY(cudaMemcpyAsync(P->x, x_h, P->n_vars * 8, cudaMemcpyDeviceToDevice, P->stream));
    else TAD_CUDA_TRY(cudaMemcpyAsync(P->x, x_h, P->n_vars * 8, cudaMemcpyHostToDevice, P->stream));
    // in mixed precision the Hessian is evaluated in FP32 and returned widened to double
    const int prec = mode >= TAD_MODE_HESSIAN ? P->precision : TAD_PREC_FP64;
    s = eval_full(*P, P->x, mode, eps, prec);
    if (s != TAD_OK) return s;
    TAD_CUDA_TRY(cudaMemcpyAsync(&P->hs->f, &P->ds->f, sizeof(double), cudaMemcpyDeviceToHost, P->stream));
    if (g_h && mode >= TAD_MODE_GRADIENT)
        TAD_CUDA_TRY(cudaMemcpyAsync(g_h, P->g, P->n_vars * 8, x_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, P->stream));
    if (H_h && mode >= TAD_MODE_HESSIAN)
    {
        launch_bsr_to_csr(*P, P->csr_tmp, prec);
        TAD_CUDA_TRY(cudaMemcpyAsync(H_h, P->csr_tmp, P->nb * P->d * P->d * 8,
                                     x_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, P->stream));
    }
    s = check_device_error(*P);   // synchronises
    if (s != TAD_OK) return s;
    *f = P->hs->f;
    return TAD_OK;
}

TAD_API tad_status tad_eval(tad_problem* P, const double* x_h, double* f)
{
    return eval_host(P, x_h, TAD_MODE_VALUE, 0.0, f, nullptr, nullptr, false);
}
TAD_API tad_status tad_eval_with_gradient(tad_problem* P, const double* x_h, double* f, double* g_h)
{
    return eval_host(P, x_h, TAD_MODE_GRADIENT, 0.0, f, g_h, nullptr, false);
}
TAD_API tad_status tad_eval_with_derivatives(tad_problem* P, const double* x_h, double* f, double* g_h, double* H_h)
{
    return eval_host(P, x_h, TAD_MODE_HESSIAN, 0.0, f, g_h, H_h, false);
}
TAD_API tad_status tad_eval_with_hessian_proj(tad_problem* P, const double* x_h, double eps, double* f, double* g_h, double* H_h)
{
    return eval_host(P, x_h, TAD_MODE_HESSIAN_PROJ, eps, f, g_h, H_h, false);
}
TAD_API tad_status tad_eval_d(tad_problem* P, const double* x_d, double* f)
{
    return eval_host(P, x_d, TAD_MODE_VALUE, 0.0, f, nullptr, nullptr, true);
}
TAD_API tad_status tad_eval_with_hessian_proj_d(tad_problem* P, const double* x_d, double eps, double* f, double* g_d, double* H_d)
{
    return eval_host(P, x_d, TAD_MODE_HESSIAN_PROJ, eps, f, g_d, H_d, true);
}

TAD_API tad_status tad_launch_count(tad_problem* P, int64_t* n)
{
    if (!P || !n) return fail(TAD_ERR_ARG, "NULL argument");
    *n = P->n_launches;
    return TAD_OK;
}

TAD_API tad_status tad_get_stream(tad_problem* P, void** stream)
{
    if (!P || !stream) return fail(TAD_ERR_ARG, "NULL argument");
    *stream = (void*)P->stream;
    return TAD_OK;
}

TAD_API tad_status tad_last_solve_stats(tad_problem* P, double* ms4, int64_t* pcg_iters, int64_t* ls_trials)
{
    if (!P) return fail(TAD_ERR_ARG, "NULL problem");
    if (ms4) for (int i = 0; i < 4; ++i) ms4[i] = P->ms_stage[i];
    if (pcg_iters) *pcg_iters = P->pcg_iters_total;
    if (ls_trials) *ls_trials = P->ls_trials_total;
    return TAD_OK;
}

} // extern "C"
