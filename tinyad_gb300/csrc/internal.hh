/*
 * Library internals shared by the C-ABI translation units.
 *
 * HBM layout of one problem (n = d * n_handles variables, interleaved x[d*v+i]):
 *   per term:  rec[n_elem][N] int32   recorded access order (-1 = unused slot)
 *              vtx/prm                 built-in energies' vertex lists / params
 *   element outputs, all terms concatenated (term offsets in units below):
 *              ef[n_elem_total]                 double, element energies
 *                                              (x LS_BATCH in line-search mode)
 *              eg[n_slots_total][d]             double, element gradient slots
 *              eH[n_pairs_total][d][d]          double (FP64) or float (mixed)
 *   pattern (built once, like LinearSolver's analyzePattern, LinearSolver.hh:12-19):
 *              bptr[n_handles+1], bcol[nb]      BSR block rows (d x d blocks)
 *              diag[n_handles]                  BSR index of each diagonal block
 *              cptr[nb+1], cidx[ncontrib]       per block: element pair blocks in
 *                                              element order (bit 31 = transposed)
 *              gptr[n_handles+1], gidx[...]     per handle: element slots
 *   assembled: g[n] double, H[nb][d][d] double (plain) / float (mixed)
 *   solver:    r, z, p, Ap, dx [n] double (plain) / float (mixed inner PCG),
 *              Dinv[n_handles][d][d]
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/tad.h"

namespace tadlib {

constexpr int LS_BATCH = 8;        // trial step sizes evaluated per launch
constexpr int RED_BLOCKS = 608;    // 4 x 152 SMs: fixed grid of the reductions
/* grid of the PCG SpMV: 8 x 152 SMs x 256 threads = 2048 threads per SM,
   full occupancy at <= 32 registers, so each SM keeps as many block-row
   gathers in flight as it can (the vector-update kernel stays on the
   reduction grid: measured faster there) */
constexpr int PCG_BLOCKS = 1216;
constexpr int RED_THREADS = 256;
/* blocks of a kernel resident on the device at once (threads per block,
   static shared memory), for grid-stride kernels that should run as one
   wave; the caller computes it once per kernel */
template <typename K>
inline unsigned resident_grid(K kernel, int threads)
{
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0);
    return (unsigned)(per > 0 ? per : 1) * (unsigned)(sms > 0 ? sms : 1);
}
/* mixed-precision solves at least this loose are one FP32 PCG pass, with no
   FP64 refinement */
constexpr double MIXED_LOOSE_TOL = 1e-4;
/* internal status of pcg_solve under pcg_async: the first iteration is
   enqueued and not yet checked */
constexpr tad_status PCG_PENDING = (tad_status)1000;

void set_error(const std::string& msg);

#define TAD_CUDA_TRY(expr)                                                          \
    do {                                                                            \
        cudaError_t _e = (expr);                                                    \
        if (_e != cudaSuccess) {                                                    \
            tadlib::set_error(std::string("CUDA error: ") + cudaGetErrorString(_e)   \
                              + " at " + __FILE__ + ":" + std::to_string(__LINE__)); \
            return TAD_ERR_CUDA;                                                    \
        }                                                                           \
    } while (0)

struct Term
{
    int energy = -1;                 // tad_energy, or -1 for a custom functor
    int N = 0;
    int64_t n_elem = 0;
    int n_params = 0;
    std::vector<int32_t> vtx_h;      // built-in: element vertex handles
    int32_t* vtx_d = nullptr;
    double* prm_d = nullptr;
    int32_t* rec_d = nullptr;        // recorded access order
    std::vector<int32_t> rec_h;
    tad_term_eval_fn fn = nullptr;
    void* user = nullptr;
    int64_t elem_off = 0, slot_off = 0, pair_off = 0;
    int M = 0;                       // vector terms: residuals per element (0: scalar term)
    int64_t out_off = 0, jac_off = 0, hv_off = 0;   // offsets into the residual buffers
};

/* device-side scalars of one problem */
struct DevScalars
{
    double f;            // energy at x
    double f_prev;       // energy before an adopted line-search step (k_ls_select)
    double f_trial[LS_BATCH];
    double dg;           // d . g
    double alpha, beta, rz, rz_new, rr, bb, pAp;
    double tol2;         // (rel_tol * |b|)^2
    int32_t done;        // PCG converged / stopped
    int32_t breakdown;   // non-positive curvature
    int32_t iters;       // PCG iterations
    int32_t max_iters;   // PCG iteration cap
    int32_t ls_choice;   // index of accepted trial in the batch, -1 none
    double ls_f;         // accepted energy
    double ls_s;         // accepted step
    double decrement;    // -0.5 d.g
    double gg;           // g.g
    int32_t spec_ok;     // Newton: the PCG is done and x is the state the carried derivatives belong to
};

/* one level of the smoothed-aggregation AMG hierarchy (amg.cu); level 0
   borrows the problem's pattern and values.  Values and vectors are sized for
   FP64 and used in the PCG's precision. */
struct AmgLevel
{
    int64_t n = 0, nb = 0;
    int32_t *bptr = nullptr, *bcol = nullptr, *diag = nullptr;   // this level's matrix
    void* A = nullptr;                       // its values (level 0: the problem's H)
    int64_t max_row = 0;                     // longest block row
    void* dl1 = nullptr;                     // inverted l1 blocks (the smoother)
    void *r = nullptr, *x = nullptr, *res = nullptr, *w = nullptr;   // V-cycle vectors (w: coarsest-level scratch)
    // transfer to the next level (all but the coarsest)
    int64_t nc = 0, np = 0, nq = 0;
    int32_t *pptr = nullptr, *pcol = nullptr, *pslot = nullptr, *pdiag = nullptr;   // P pattern
    int32_t *qptr = nullptr, *qcol = nullptr;                                     // Q = A P pattern
    int32_t *qlptr = nullptr, *qla = nullptr, *qlp = nullptr;                      // per Q block: (A, P) products
    int32_t *qrow = nullptr, *qpb = nullptr;                                      // per Q block: its row, its P block (-1)
    int32_t *tptr = nullptr, *tu = nullptr, *tp = nullptr;                        // transposed P lists
    double* cscale = nullptr;                // per aggregate 1 / sqrt(size)
    void *Pv = nullptr, *Qv = nullptr;       // P and Q values
    void* Rv = nullptr;                      // R = P - S Q on Q's pattern (the post-smoothing's operator)
};

struct Problem
{
    std::vector<AmgLevel> amg;       // smoothed-aggregation AMG hierarchy (pattern built at finalisation)
    int64_t amg_solves = 0;          // solves that used it (statistics)
    bool amg_sticky = false;         // the last solve needed the V-cycle: the next one switches after its first iteration
    bool in_newton = false;          // solves of the Newton loop (the only ones that use amg_sticky)
    int amg_last_chunks = 0;         // captured V-cycle chunks the last V-cycle solve of the Newton loop needed
    bool amg_values_ready = false;   // values computed for the current H

    int kind = 0;                    // 0: empty, 1: scalar terms, 2: vector terms (sum of squares)
    int64_t n_outputs_total = 0;     // vector problems: residuals
    int64_t jac_size = 0, hv_size = 0;
    double* vr = nullptr;            // residuals [n_outputs]
    double* vJ = nullptr;            // residual gradients, per term [n_elem][M][k]
    double* vHv = nullptr;           // packed residual Hessians, per term [n_elem][M][k(k+1)/2]
    int vec_outputs = 0;             // which of vr / vJ / vHv the next evaluation fills (0..3)
    std::vector<int32_t> jptr_h, jcol_h;   // Jacobian CSR pattern (n_outputs x n_vars)
    int32_t* jmap = nullptr;         // Jacobian CSR value k -> index into vJ

    int d = 0;
    int64_t n_handles = 0, n_vars = 0;
    tad_settings settings{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<Term> terms;
    bool finalized = false;
    int precision = TAD_PREC_FP64;

    int64_t n_elem_total = 0, n_slots_total = 0, n_pairs_total = 0;
    double* ef = nullptr;
    double* eg = nullptr;
    void* eH = nullptr;
    size_t eH_bytes = 0;
    uint32_t* proj_list = nullptr;   // largest term's n_elem + 1: elements left for the general projection

    // pattern
    int64_t nb = 0, ncontrib = 0, ninc = 0;
    std::vector<int32_t> bptr_h, bcol_h;
    int32_t *bptr = nullptr, *bcol = nullptr, *diag = nullptr;
    int32_t *cptr = nullptr, *cidx = nullptr;
    int32_t *gptr = nullptr, *gidx = nullptr;

    // assembled quantities
    double* x = nullptr;
    double* g = nullptr;
    void* H = nullptr;         // nb*d*d, double or float
    // sliced-ELL copy of H for the SpMVs: block rows in slices of 32; slot
    // sptr[s] + j * 32 + (u mod 32) holds the j-th block of row u of slice s
    // (zero blocks pad rows shorter than their slice's longest), so a warp's
    // 32 rows read their j-th blocks and column ids as contiguous ranges
    int64_t n_slots = 0;
    int32_t *sptr = nullptr, *scol = nullptr;   // slices + 1 / slots
    int32_t *spos = nullptr, *sdiag = nullptr;  // per BSR block / per block row: its slot
    void* Hs = nullptr;                          // n_slots*d*d, as H (null: no copy, CSR SpMVs)
    const void* Hs_of = nullptr;                 // the buffer Hs copies (H as allocated; solves may swap H)
    double* H64 = nullptr;     // FP64 copy for mixed-mode refinement residuals (optional)
    double* csr_tmp = nullptr; // CSR-ordered values for export

    // solver work
    double *r = nullptr, *z = nullptr, *p = nullptr, *Ap = nullptr, *dx = nullptr, *dinv = nullptr;
    float *r32 = nullptr, *z32 = nullptr, *p32 = nullptr, *Ap32 = nullptr, *dx32 = nullptr, *dinv32 = nullptr;
    double *rhs = nullptr, *res = nullptr;
    double* x_trial = nullptr;   // Newton: the speculative full-step state x + d (n_vars, allocated on first use)
    // tad_term_eval_args.active_d of element launches: NULL, or a device int
    // that is 0 when the launch has nothing to do (batched line searches whose
    // meshes all accepted; the Newton loop's speculative evaluation before the
    // PCG has converged)
    const int32_t* launch_guard = nullptr;
    // Newton state kept across solver calls: the last call's final x and,
    // when its last iteration took the speculative trial, the derivatives
    // assembled there (valid for spec_eps / spec_prec until any other
    // evaluation or a settings change)
    double* last_x = nullptr;
    bool last_x_valid = false;
    bool spec_valid = false;
    double spec_eps = 0.0;
    int spec_prec = -1;
    int streak = 0;                  // consecutive calls that continued from the previous call's x
    int32_t* diff_flag = nullptr;    // device: x differs from last_x
    int32_t* diff_flag_h = nullptr;  // pinned mirror
    cudaStream_t stream2 = nullptr;  // side stream: host copies of x and the continuation test beside the compute
    cudaEvent_t ev_in = nullptr, ev_xt = nullptr, ev_out = nullptr;
    bool defer_fp32 = false;     // Newton asks a loose mixed solve to leave its solution in dx32 ...
    bool solution_in_dx32 = false;   // ... and the solve says it did (P.dx not written)
    bool pcg_async = false;      // Newton: return PCG_PENDING after the first iteration, without a host check
    bool pcg_resume = false;     // Newton: continue a PCG_PENDING solve (its first check is in P.hs)
    double* steps = nullptr;   // LS_BATCH trial step sizes (device)
    double* steps_seq = nullptr;   // the line search's whole step sequence (device), for steps_key
    int steps_seq_cap = 0;
    double steps_key[3] = {0.0, 0.0, 0.0};   // s_max, shrink, length of the sequence in steps_seq
    double* partials = nullptr;
    unsigned* counters = nullptr;
    DevScalars* ds = nullptr;
    DevScalars* hs = nullptr;  // pinned mirror
    int32_t* err = nullptr;
    int32_t* err_h = nullptr;  // pinned

    // captured PCG iteration graphs (chunk of iterations)
    cudaGraphExec_t pcg_graph = nullptr;
    cudaGraphExec_t amg_graph = nullptr;     // chunk of AMG-preconditioned CG iterations
    const void* pcg_graph_H = nullptr;       // the Hessian buffer each graph reads
    const void* amg_graph_H = nullptr;
    void* Hd = nullptr;                      // FP64 copy of an FP32 Hessian (tight mixed solves)
    double* corr = nullptr;                  // FP64 correction of a tight mixed solve
    int amg_graph_prec = -1;
    const void* amg_graph_x = nullptr;
    int64_t amg_graph_launches = 0;          // kernels in one replay of amg_graph
    int pcg_graph_chunk = 0;
    int pcg_graph_prec = -1;
    const void* pcg_graph_x = nullptr;

    // stats of the last solve
    double ms_stage[4] = {0, 0, 0, 0};
    int64_t pcg_iters_total = 0, ls_trials_total = 0;
    double g0_norm = 0.0;      // |g| at the first iteration of the last solve
    int64_t n_launches = 0;    // kernels launched by this problem (cumulative)
    cudaEvent_t ev[8] = {};
    // Newton stage timing: 5 events per iteration, read after the loop (no
    // per-iteration event wait on the host's critical path)
    static constexpr int STAGE_ITERS = 256;
    std::vector<cudaEvent_t> stage_ev;
    bool timing = false;
};

// ---- problem.cu
tad_status ensure_finalized(Problem& P);
tad_status check_device_error(Problem& P);

// ---- builtin_*.cu: launch a built-in energy term for one evaluation mode
tad_status launch_builtin(Problem& P, Term& T, const tad_term_eval_args& a);
tad_status launch_builtin_vec(Problem& P, Term& T, const tad_term_eval_args& a);
tad_status launch_builtin_tri(Problem& P, Term& T, const tad_term_eval_args& a);
tad_status launch_builtin_tet(Problem& P, Term& T, const tad_term_eval_args& a);
tad_status launch_builtin_misc(Problem& P, Term& T, const tad_term_eval_args& a);

// ---- eval.cu
/* evaluate all terms in `mode` at x (device) into the element buffers */
tad_status eval_elements(Problem& P, int mode, const double* x, double eps, int precision,
                         const double* dir = nullptr, int n_steps = 0);
/* assemble element buffers -> f (device scalar ds->f), g, H */
/* f (into f_dst, default ds->f), gradient and Hessian from the element
   buffers; newton_rhs: the gradient assembly also writes rhs = -g and ds->gg */
tad_status assemble(Problem& P, bool gradient, bool hessian, int precision, double* f_dst = nullptr, bool newton_rhs = false);
/* full f/g/H evaluation at device x */
tad_status eval_full(Problem& P, const double* x, int mode, double eps, int precision);

// ---- kernels (kernels.cu)
void launch_reduce_f(Problem& P, int n_rows, double* out);      // sums ef rows into out[row]
/* g from the element gradient slots, in element order; mixed precision sums
   in double-float.  pairs: the slots hold double-float pairs (what the
   mixed second-order element kernels write) */
void launch_assemble_grad(Problem& P, int precision = TAD_PREC_FP64, bool pairs = false);
/* the same, also rhs = -g and ds->gg = g.g (Newton right-hand side) */
void launch_assemble_grad_newton(Problem& P, int precision, bool pairs);
void launch_assemble_hess(Problem& P, int precision);
void launch_bsr_to_csr(Problem& P, double* out, int precision);
void launch_zero(double* p, int64_t n, cudaStream_t s);

// ---- solver.cu
void add_identity(Problem& P, double w, int precision);   // H += w I (assembled H)
tad_status amg_build(Problem& P);                         // the hierarchy's patterns (once per problem)
tad_status amg_prepare(Problem& P, int precision);        // hierarchy (if not built) + values for the current H
/* CG under the V-cycle, on P.stream: mode 0 restarts from the current (xs, r)
   (z = V(r), p = Ap = 0, beta = 0); mode 1 is the step after the fused SpMV
   (x += alpha p, r -= alpha Ap with the stop test, z = V(r), beta) */
void amg_apply(Problem& P, int precision, int mode, void* xs, void* r, void* z, void* p, void* Ap);
void amg_free(Problem& P);
int amg_levels(const Problem& P);
tad_status prepare_solver_graphs(Problem& P);              // capture the Newton loop's PCG graphs (finalisation)
tad_status pcg_solve(Problem& P, const double* b, double* xsol, double w_identity, int precision,
                     double rel_tol, int max_iters, int* iters_out);
/* f_on_device: the energy at x is already in ds->f (f is then ignored);
   t_start > 0 resumes the trial sequence there with ds->dg already set;
   stop_decrement > 0: if -d.g/2 < stop_decrement, x is left as it is and
   *stopped is set (the Newton loop's stopping test, taken before the step) */
tad_status line_search_device(Problem& P, double* x, const double* d, double f, double s_max,
                              bool* found, double* f_out, int* trials, bool f_on_device = false, int t_start = 0,
                              double stop_decrement = 0.0, bool* stopped = nullptr);
/* x_in_h / x_out_h (host API): x is copied in from and out to these host
   buffers by the solve itself, overlapped with the compute where it can */
tad_status newton_solve(Problem& P, double* x_d, int n_iters, double eps, double stop_decrement,
                        double* f_hist, int* iters_done, const double* x_in_h = nullptr, double* x_out_h = nullptr);

} // namespace tadlib

struct tad_problem : public tadlib::Problem {};
