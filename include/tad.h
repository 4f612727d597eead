/*
 * tad.h -- C ABI of the GB300 sparse per-element derivative library.
 *
 * One opaque problem object stands for one TinyAD ScalarFunction: a set of
 * d-dimensional variable handles plus a list of objective terms, each a set
 * of elements of fixed valence N evaluated by a per-element energy.  All
 * entry points take plain pointers and sizes; "_h" buffers are host memory,
 * "_d" buffers are device memory of the current CUDA device.
 *
 * Reference interface each entry point replaces (TinyAD, MIT licence):
 *   tad_problem_create        ScalarFunction ctor / scalar_function<d>(range)
 *                             include/TinyAD/Detail/ScalarFunctionImpl.hh:47-61, :418-442
 *   tad_add_elements          ScalarFunction::add_elements<N>(range, lambda)
 *                             include/TinyAD/Detail/ScalarFunctionImpl.hh:63-100
 *   tad_add_elements_custom   the same, for a user functor compiled by the C++
 *                             front end (include/tad/ScalarFunction.cuh)
 *   tad_eval                  ScalarFunction::eval / operator()
 *                             include/TinyAD/Detail/ScalarFunctionImpl.hh:256-282
 *   tad_eval_with_gradient    ScalarFunction::eval_with_gradient
 *                             include/TinyAD/Detail/ScalarFunctionImpl.hh:284-314
 *   tad_eval_with_derivatives ScalarFunction::eval_with_derivatives / eval_hessian
 *                             include/TinyAD/Detail/ScalarFunctionImpl.hh:316-376
 *   tad_eval_with_hessian_proj ScalarFunction::eval_with_hessian_proj
 *                             include/TinyAD/Detail/ScalarFunctionImpl.hh:378-416
 *   tad_hessian_pattern       the index arrays of the returned Eigen::SparseMatrix
 *                             (outerIndexPtr/innerIndexPtr; H is symmetric so the
 *                             CSR arrays here equal Eigen's CSC arrays)
 *   tad_newton_direction      newton_direction(g, H, solver)
 *                             include/TinyAD/Utils/NewtonDirection.hh:25-65
 *   tad_newton_direction_reduced_basis  newton_direction_reduced_basis(g, H, B, solver)
 *                             include/TinyAD/Utils/NewtonDirection.hh:76-123
 *   tad_add_vector_elements*, tad_vec_*, tad_eval_sum_of_squares_with_derivatives
 *                             VectorFunction (include/TinyAD/VectorFunction.hh,
 *                             Detail/VectorObjectiveTerm.hh)
 *   tad_gauss_newton_direction gauss_newton_direction(r, J, solver, w)
 *                             include/TinyAD/Utils/GaussNewtonDirection.hh:24-64
 *   tad_line_search           line_search(x, d, f, g, func)
 *                             include/TinyAD/Utils/LineSearch.hh:26-65
 *   tad_newton_decrement      newton_decrement(d, g)
 *                             include/TinyAD/Utils/NewtonDecrement.hh:20-26
 *   tad_newton_solve          the Projected-Newton loop users write around the
 *                             three calls above (tests/NewtonTest.cc:69-75)
 *   tad_adjoint_rest_gradient no reference counterpart (adjoint extension)
 *   tad_batch_*               no reference counterpart (batched extension)
 *
 * Errors: every entry point returns a tad_status; tad_last_error_message()
 * gives the text for the calling thread.  The reference throws
 * std::runtime_error (include/TinyAD/Utils/Out.hh:73-79); the C++ front end
 * turns a non-OK status back into that exception.  A problem stays usable
 * after an error (tests/ExceptionTest.cc:8-53).
 */
#ifndef TAD_H
#define TAD_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define TAD_API __declspec(dllexport)
#else
#define TAD_API __attribute__((visibility("default")))
#endif

typedef enum tad_status {
    TAD_OK = 0,
    TAD_ERR_ARG = 1,          /* invalid argument (sizes, handles, null pointers) */
    TAD_ERR_NONFINITE = 2,    /* non-finite input or non-finite derivative */
    TAD_ERR_PCG_NOCONV = 3,   /* linear solve did not reach its tolerance */
    TAD_ERR_LS_FAIL = 4,      /* warning: line search found no decrease, x kept */
    TAD_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
    TAD_ERR_CUDA = 6,         /* CUDA runtime error */
    TAD_ERR_STATE = 7,        /* call not valid in the problem's current state */
    TAD_ERR_TOO_MANY_VARS = 8 /* element accessed more handles than its valence */
} tad_status;

/* Built-in per-element energies (params are per element, doubles). */
typedef enum tad_energy {
    /* d=2, N=3: params [Mr00 Mr10 Mr01 Mr11 w] (Mr column-major = rest edge
       matrix [b-a, c-a]).  E = w * (|M Mr^-1|_F^2 + |Mr M^-1|_F^2), +inf if
       det M <= 0.  Same lambda as tests/NewtonTest.cc:28-44. */
    TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI = 0,
    /* d=3, N=4: params [Mr (3x3 column-major) w], 3D analogue. */
    TAD_ENERGY_SYMMETRIC_DIRICHLET_TET = 1,
    /* any d, N=1: params [target(d) w].  E = w * |target - p|^2
       (tests/NewtonTest.cc:48-55). */
    TAD_ENERGY_POSITION_PENALTY = 2,
    /* any d, N: params [A (k*k, row-major) b (k) c], k = d*N.
       E = sum_ij A_ij x_i x_j + sum_i b_i x_i + c over the element's
       variables in access order (the quadratics of tests/ScalarFunctionTest.cc). */
    TAD_ENERGY_QUADRATIC = 3,
    /* any d, N=3: params [w].  E = w * (|b-a|^2 + |c-b|^2 + |a-c|^2)
       (the Laplacian test of tests/DynamicElementsTest.cc:60-91 with w=1/4). */
    TAD_ENERGY_DIRICHLET_TRI = 4,
    TAD_ENERGY_COUNT_ = 5
} tad_energy;

/* Built-in residual functors of vector terms (VectorFunction). */
typedef enum tad_vector_energy {
    /* d=2, N=3, 8 outputs: params as TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI.
       r = sqrt(w) [J00 J01 J10 J11 Ji00 Ji01 Ji10 Ji11] with J = M Mr^-1,
       Ji = Mr M^-1 (+inf residuals if det M <= 0), so sum r^2 is the
       symmetric Dirichlet energy (tests/GaussNewtonTest.cc:33-66). */
    TAD_VEC_SYMMETRIC_DIRICHLET_TRI = 0,
    /* any d, N=1, d outputs: params [target(d) w].  r = sqrt(w) (target - p)
       (tests/GaussNewtonTest.cc:67-74). */
    TAD_VEC_POSITION = 1
} tad_vector_energy;

typedef enum tad_precision {
    TAD_PREC_FP64 = 0,   /* plain drop-in: everything in double */
    TAD_PREC_MIXED = 1   /* FP32 element Hessians, projection and PCG; FP64
                            determinant/inverse, line-search energy and
                            iterative-refinement residuals */
} tad_precision;

typedef struct tad_settings {
    int precision;            /* tad_precision */
    int pcg_max_iters;        /* per linear solve (default 1000) */
    double pcg_rel_tol;       /* relative residual target (default 1e-10) */
    int refine_max_iters;     /* mixed mode: iterative-refinement passes (default 4) */
    double refine_rel_tol;    /* mixed mode: FP64 residual target (default 1e-10) */
    int ls_max_iters;         /* line search trials (reference default 64) */
    double ls_shrink;         /* 0.8 */
    double ls_armijo;         /* 1e-4 */
    int forcing;              /* Newton loop: 0 = fixed pcg_rel_tol; 1 = inexact
                                 Newton, tol_k = max(pcg_rel_tol,
                                 min(0.5, sqrt(|g_k| / |g_0|))), g_0 = the
                                 gradient at the first Newton iteration after
                                 tad_problem_create / tad_problem_set_settings */
    int verbose;
    int preconditioner;       /* 0 = block Jacobi; 1 (default) = block Jacobi, and an
                                 FP64 solve whose residual is still more than 4x
                                 above its target after 9 iterations restarts with
                                 conjugate gradients preconditioned by an
                                 aggregation-AMG V-cycle (FP32 solves of mixed
                                 precision keep block Jacobi) */
} tad_settings;

typedef struct tad_problem tad_problem;

/* Fill *s with the defaults above. */
TAD_API void tad_settings_default(tad_settings* s);

TAD_API const char* tad_last_error_message(void);
TAD_API const char* tad_version(void);

/* Create a problem with n_handles variable handles of dimension var_dim
   (n_vars = var_dim * n_handles, interleaved x[d*v + i]).  Uses the current
   CUDA device. */
TAD_API tad_status tad_problem_create(int var_dim, int64_t n_handles,
                                      const tad_settings* settings,
                                      tad_problem** out);
TAD_API tad_status tad_problem_destroy(tad_problem* p);
TAD_API tad_status tad_problem_set_settings(tad_problem* p, const tad_settings* s);
TAD_API int64_t tad_n_vars(const tad_problem* p);

/* Add n_elem elements of valence N, each naming N variable handles in the
   order its energy accesses them (handles_h: n_elem*N int32, host), with
   n_params doubles per element (params_h: n_elem*n_params, host). */
TAD_API tad_status tad_add_elements(tad_problem* p, int energy, int valence,
                                    int64_t n_elem, const int32_t* handles_h,
                                    const double* params_h, int n_params);

/* User-functor terms (the C++ front end).  The callback evaluates all
   elements of the term on the library's stream and writes per-element
   outputs into library-owned device buffers; see tad_term_eval_args. */
typedef struct tad_term_eval_args {
    int mode;                 /* tad_eval_mode */
    int precision;            /* tad_precision of the outputs */
    int64_t n_elem;
    int valence;
    int var_dim;
    const double* x_d;        /* current x (device, n_vars) */
    const double* dir_d;      /* line search: direction (device) */
    const double* steps_d;    /* line search: n_steps trial step sizes */
    int n_steps;
    int64_t f_row_stride;     /* line search: trial j writes out_f_d + j*f_row_stride */
    double proj_eps;
    const int32_t* handles_d; /* recorded access order, n_elem*N, -1 = unused slot */
    void* out_f_d;            /* double[n_elem] (or [n_steps][n_elem]) */
    void* out_g_d;            /* [n_elem][N*d] in output precision */
    void* out_H_d;            /* [n_elem][N(N+1)/2 slot pairs][d][d] */
    int32_t* record_d;        /* TAD_MODE_RECORD: write accessed handles here */
    int32_t* error_d;         /* device error word (OR in TAD_DEVERR_* bits) */
    void* stream;             /* cudaStream_t */
    /* vector terms (VectorFunction) only; 0 / NULL for scalar terms */
    int n_outputs;            /* residuals per element, M */
    double* out_r_d;          /* [n_elem][M] residuals, or NULL */
    double* out_J_d;          /* [n_elem][M][N*d] residual gradients in local slot order, or NULL */
    double* out_Hv_d;         /* [n_elem][M][k(k+1)/2] packed residual Hessians, k = N*d, or NULL */
    /* HESSIAN_PROJ: device scratch of n_elem + 1 uint32 (library-owned): the
       element kernels list there the elements whose Hessian is not
       translation invariant, which then get the general projection */
    uint32_t* proj_list_d;
    /* LINESEARCH, HESSIAN, HESSIAN_PROJ: NULL, or a device int read at the
       start of the launch; 0 means the launch has nothing to do (every group
       of a batched line search has accepted a step; a speculative evaluation
       whose linear solve has not converged) and it returns without work or
       outputs */
    const int32_t* active_d;
} tad_term_eval_args;

typedef enum tad_eval_mode {
    TAD_MODE_VALUE = 0,       /* f only */
    TAD_MODE_GRADIENT = 1,    /* f, g */
    TAD_MODE_HESSIAN = 2,     /* f, g, H */
    TAD_MODE_HESSIAN_PROJ = 3,/* f, g, PSD-projected H */
    TAD_MODE_LINESEARCH = 4,  /* f at x + s_j * dir for j < n_steps */
    TAD_MODE_RECORD = 5,      /* record first-access handle order */
    TAD_MODE_VEC_JACOBIAN = 6,    /* vector terms: residuals and their gradients */
    TAD_MODE_VEC_DERIVATIVES = 7  /* vector terms: residuals, gradients and Hessians */
} tad_eval_mode;
/* For vector terms the scalar modes refer to the sum of squares f = sum_i r_i^2:
   VALUE and LINESEARCH write f per element, GRADIENT adds g = 2 J^T r, and
   HESSIAN / HESSIAN_PROJ add the Gauss-Newton blocks 2 J_e^T J_e (PSD, so the
   projection has nothing to do). */

typedef int (*tad_term_eval_fn)(void* user, const tad_term_eval_args* args);

/* A term of n_elem elements of valence 1..64 evaluated by a caller-supplied
   device functor (fn launches the element kernels for args->mode; the C++
   front end instantiates them from a lambda).  The library records each
   element's access order with one TAD_MODE_RECORD call when the sparsity
   pattern is built. */
TAD_API tad_status tad_add_elements_custom(tad_problem* p, int valence,
                                           int64_t n_elem,
                                           tad_term_eval_fn fn, void* user);

/* Build the sparsity pattern now (otherwise done by the first eval). */
TAD_API tad_status tad_finalize(tad_problem* p);

/* Number of non-zeros of the assembled Hessian (explicit zeros kept, so
   nnz = union of the element blocks, as Eigen's setFromTriplets keeps them). */
TAD_API tad_status tad_hessian_nnz(tad_problem* p, int64_t* nnz);
/* CSR arrays of the pattern: outer (n_vars+1) and inner (nnz), int32, host. */
TAD_API tad_status tad_hessian_pattern(tad_problem* p, int32_t* outer_h, int32_t* inner_h);

/* Evaluations (host buffers).  g_h: n_vars doubles.  H_values_h: nnz doubles
   in the order of tad_hessian_pattern (may be NULL to skip the copy). */
TAD_API tad_status tad_eval(tad_problem* p, const double* x_h, double* f);
TAD_API tad_status tad_eval_with_gradient(tad_problem* p, const double* x_h,
                                          double* f, double* g_h);
TAD_API tad_status tad_eval_with_derivatives(tad_problem* p, const double* x_h,
                                             double* f, double* g_h, double* H_values_h);
TAD_API tad_status tad_eval_with_hessian_proj(tad_problem* p, const double* x_h,
                                              double proj_eps, double* f,
                                              double* g_h, double* H_values_h);
/* Device-pointer variants (zero copy). */
TAD_API tad_status tad_eval_d(tad_problem* p, const double* x_d, double* f);
TAD_API tad_status tad_eval_with_hessian_proj_d(tad_problem* p, const double* x_d,
                                                double proj_eps, double* f,
                                                double* g_d, double* H_values_d);

/* d = -(H + w I)^-1 g with H the Hessian at x -- PSD-projected with proj_eps
   if `projected` (eval_with_hessian_proj), else exact (eval_with_derivatives)
   -- solved by block-Jacobi PCG on the device (w_identity >= 0).
   Returns TAD_ERR_PCG_NOCONV if the tolerance is not met (d then holds the
   last iterate). */
TAD_API tad_status tad_newton_direction(tad_problem* p, const double* x_h, int projected,
                                        double proj_eps, double w_identity,
                                        double* d_h, double* f, double* g_h);

/* ---- vector functions (include/TinyAD/VectorFunction.hh) -----------------
   A problem holds either scalar terms (tad_add_elements*) or vector terms
   (tad_add_vector_elements*), whose functors return n_outputs residuals per
   element.  On a vector problem the scalar entry points act on the sum of
   squares f = sum_i r_i^2 (tad_eval = eval_sum_of_squares; gradient 2 J^T r;
   the Hessian entry points and tad_newton_solve use the Gauss-Newton matrix
   2 J^T J, so tad_newton_solve runs Gauss-Newton with the Armijo line search
   on f).  Residuals are numbered term by term, element by element
   (Detail/VectorObjectiveTerm.hh:160-215). */
TAD_API tad_status tad_add_vector_elements(tad_problem* p, int energy, int valence, int n_outputs,
                                           int64_t n_elem, const int32_t* element_vertices_h,
                                           const double* params_h, int n_params);
TAD_API tad_status tad_add_vector_elements_custom(tad_problem* p, int valence, int n_outputs, int64_t n_elem,
                                                  tad_term_eval_fn fn, void* user);
/* number of residuals (VectorFunction::n_outputs) */
TAD_API int64_t tad_n_outputs(const tad_problem* p);
/* VectorFunction::eval: r[n_outputs] */
TAD_API tad_status tad_vec_eval(tad_problem* p, const double* x_h, double* r_h);
/* the Jacobian's CSR pattern (n_outputs x n_vars, columns sorted per row):
   the variables of each residual's element, as the reference's triplets
   (VectorObjectiveTerm.hh:214-221) */
TAD_API tad_status tad_vec_jacobian_nnz(tad_problem* p, int64_t* nnz);
TAD_API tad_status tad_vec_jacobian_pattern(tad_problem* p, int32_t* outer, int32_t* inner);
/* VectorFunction::eval_with_jacobian: r and the CSR values of J */
TAD_API tad_status tad_vec_eval_with_jacobian(tad_problem* p, const double* x_h, double* r_h, double* J_values_h);
/* VectorFunction::eval_with_derivatives: r, J and the residual Hessians as
   triplets, output i owning [H_ptr[i], H_ptr[i+1]) (tad_vec_hessians_nnz
   entries in all) */
TAD_API tad_status tad_vec_hessians_nnz(tad_problem* p, int64_t* nnz);
TAD_API tad_status tad_vec_eval_with_derivatives(tad_problem* p, const double* x_h, double* r_h, double* J_values_h,
                                                 int64_t* H_ptr, int32_t* H_row, int32_t* H_col, double* H_val);
/* VectorFunction::eval_sum_of_squares_with_derivatives: f, g = 2 J^T r, r, J
   (Detail/VectorFunctionImpl.hh:271-283) */
TAD_API tad_status tad_eval_sum_of_squares_with_derivatives(tad_problem* p, const double* x_h, double* f,
                                                            double* g_h, double* r_h, double* J_values_h);
/* gauss_newton_direction(r, J, solver, w) (Utils/GaussNewtonDirection.hh:24-47)
   at x: d = -(J^T J + w I)^-1 J^T r, device PCG to pcg_rel_tol; also returns
   f and g of the sum of squares. */
TAD_API tad_status tad_gauss_newton_direction(tad_problem* p, const double* x_h, double w_identity, double* d_h,
                                              double* f, double* g_h);

/* newton_direction_reduced_basis(g, H_proj, B, solver, w)
   (include/TinyAD/Utils/NewtonDirection.hh:76-123): with g and the projected
   Hessian (proj_eps) evaluated at x, returns d = B (B^T H B + w I)^-1 (-B^T g)
   for the n_vars x m basis B given as CSR (b_outer[n_vars + 1], b_inner and
   b_values[b_outer[n_vars]], column indices in [0, m)).  The reduced system is
   solved matrix-free by conjugate gradients with the exact diagonal of
   B^T H B + w I as preconditioner, to the problem's pcg_rel_tol.  Returns
   TAD_ERR_PCG_NOCONV (d = the last iterate) if the tolerance is not met or
   the reduced system shows non-positive curvature (the reference throws
   "Linear solve failed"). */
TAD_API tad_status tad_newton_direction_reduced_basis(tad_problem* p, const double* x_h, int64_t m,
                                                      const int32_t* b_outer, const int32_t* b_inner,
                                                      const double* b_values, double proj_eps, double w_identity,
                                                      double* d_h, double* f, double* g_h);

/* Armijo backtracking from x along d: s = s_max, s *= shrink, at most
   max_iters trials; x_out = x + s d for the first s meeting
   f(x+sd) <= f + c s d.g, else x_out = x and TAD_ERR_LS_FAIL. */
TAD_API tad_status tad_line_search(tad_problem* p, const double* x_h,
                                   const double* d_h, double f, const double* g_h,
                                   double s_max, double* x_out_h, double* f_out);

/* newton_decrement(d, g) = -d.g / 2 (one half of the squared Newton
   decrement; the stopping test of the reference's Newton loop), computed on
   the device with a fixed-order reduction (bitwise reproducible).  d and g
   hold n_vars doubles: host buffers for tad_newton_decrement, device
   buffers for tad_newton_decrement_d. */
TAD_API tad_status tad_newton_decrement(tad_problem* p, const double* d_h, const double* g_h, double* out);
TAD_API tad_status tad_newton_decrement_d(tad_problem* p, const double* d_d, const double* g_d, double* out);

/* Run n_iters Projected-Newton iterations in place on x_h (host):
   eval_with_hessian_proj -> PCG -> Armijo line search, all on the device.
   f_hist_h (optional, n_iters+1): energy before each iteration and at the end.
   Stops early when the Newton decrement -d.g/2 < stop_decrement (if > 0):
   as in the reference's loop, the test is taken on the new direction before
   the line search, so that iteration leaves x as it is; *iters_done counts
   the steps taken and f_hist_h[*iters_done] is the final energy. */
TAD_API tad_status tad_newton_solve(tad_problem* p, double* x_h, int n_iters,
                                    double proj_eps, double stop_decrement,
                                    double* f_hist_h, int* iters_done);
/* The same on a device-resident x (no host copies). */
TAD_API tad_status tad_newton_solve_d(tad_problem* p, double* x_d, int n_iters,
                                      double proj_eps, double stop_decrement,
                                      double* f_hist_h, int* iters_done);

/* Adjoint: gradient of a loss L(x*) with respect to the 3D rest positions
   (n_handles x 3, host) of the built-in symmetric Dirichlet triangle terms,
   x* being a minimiser (x_h).  Solves H lambda = dL/dx (dLdx_h) with the
   PCG (H projected with proj_eps if `projected`, else the exact Hessian),
   then dL/drest = -(d2E/dx drest)^T lambda with per-element mixed second
   derivatives recomputed on the device.  lambda_h (n_vars) and pcg_iters
   are optional outputs.  No reference counterpart: the reference offers the
   building block (block-restricted Hessians, Scalar.hh:24) but no adjoint. */
TAD_API tad_status tad_adjoint_rest_gradient(tad_problem* p, const double* x_h, const double* dLdx_h,
                                             const double* rest_h, int projected, double proj_eps,
                                             double* dLdrest_h, double* lambda_h, int* pcg_iters);

/* ---- Batched solves: many independent meshes in one problem --------------
   No reference counterpart (TinyAD solves one ScalarFunction at a time).
   Each mesh m has n_handles[m] handles (mesh-local handles 0..n-1, x laid out
   mesh after mesh); every stage of a Newton iteration is one launch for all
   meshes, the iteration is one captured CUDA graph, and every mesh keeps its
   own energy, PCG scalars (pcg_rel_tol, at most pcg_max_iters iterations per
   Newton step), Armijo choice (16 trial steps) and step. */
typedef struct tad_batch tad_batch;
TAD_API tad_status tad_batch_create(int var_dim, int n_meshes, const int64_t* n_handles,
                                    const tad_settings* settings, tad_batch** out);
/* n_elem_per_mesh[m] elements per mesh, handles mesh-local, meshes in order */
TAD_API tad_status tad_batch_add_elements(tad_batch* b, int energy, int valence,
                                          const int64_t* n_elem_per_mesh, const int32_t* handles_h,
                                          const double* params_h, int n_params);
/* f_hist_h (optional): [n_iters + 1][n_meshes] energies */
TAD_API tad_status tad_batch_newton_solve(tad_batch* b, double* x_h, int n_iters, double proj_eps,
                                          double* f_hist_h);
TAD_API tad_status tad_batch_newton_solve_d(tad_batch* b, double* x_d, int n_iters, double proj_eps,
                                            double* f_hist_h);
/* times candidate (block rows per chunk, threads per block, blocks per SM
   of the persistent PCG) triples on the batch at x_d and keeps the fastest;
   best3 = [rows, threads, ms] */
TAD_API tad_status tad_batch_autotune(tad_batch* b, const double* x_d, double proj_eps, double* best3);
/* sets the chunking directly: chunk_rows block rows per PCG chunk (4x as many
   elements per element chunk), threads per block; the next solve recaptures */
TAD_API tad_status tad_batch_set_chunking(tad_batch* b, int chunk_rows, int threads);
/* the underlying concatenated problem (for evaluations, stats, the stream) */
TAD_API tad_status tad_batch_problem(tad_batch* b, tad_problem** p);
TAD_API tad_status tad_batch_destroy(tad_batch* b);

/* Time the main kernels once each at x_d (device), averaged over reps
   launches with CUDA events on the problem's stream: ms5 = [element Hessian
   kernels, gradient + Hessian assembly, one PCG SpMV, one PCG vector update,
   one line-search energy evaluation]. */
TAD_API tad_status tad_profile_kernels(tad_problem* p, const double* x_d, int reps, double* ms5);

/* Cumulative number of CUDA kernels the problem has launched. */
TAD_API tad_status tad_launch_count(tad_problem* p, int64_t* n);

/* The CUDA stream (cudaStream_t) all work of the problem is issued on. */
TAD_API tad_status tad_get_stream(tad_problem* p, void** stream);

/* Per-stage timing of the last tad_newton_solve[_d] call (milliseconds,
   CUDA events): [eval+project, assemble, pcg, line search], plus PCG
   iteration total.  Any pointer may be NULL. */
TAD_API tad_status tad_last_solve_stats(tad_problem* p, double* ms_stages4,
                                        int64_t* pcg_iters_total,
                                        int64_t* ls_trials_total);

/* Diagnostics: apply one operator of the device scalar tad::Scalar<1>
   (precision TAD_PREC_FP64: Double<1>; TAD_PREC_MIXED: Mixed<1>) to
   a = (val, grad, hess) and b, writing (val, grad, hess).  Op codes:
   0 -a, 1 sqrt, 2 sqr, 3 pow(a, int b.val), 4 pow(a, b.val), 5 exp, 6 log,
   7 sin, 8 cos, 9 tan, 10 asin, 11 acos, 12 atan, 13 sinh, 14 cosh, 15 tanh,
   16 fabs, 17 a+b, 18 a-b, 19 a*b, 20 a/b, 21 atan2(a,b), 22 hypot(a,b),
   23 b.val/a, 24 log2, 25 log10, 26 asinh, 27 acosh, 28 atanh, 29 a+b.val,
   30 a*b.val, 31 b.val-a, 32 a/b.val.  Replaces the operator known-answer
   tests of tests/ScalarTestUnaryOperators.cc / ScalarTestBinaryOperators.cc. */
TAD_API tad_status tad_debug_scalar_op(int op, int precision, const double* a3,
                                       const double* b3, double* out3);

/* Measured CUDA-core FMA throughput of the current device in TFLOP/s
   (precision TAD_PREC_FP64: double, TAD_PREC_MIXED: float); the roofline
   denominator of the element kernels. */
TAD_API tad_status tad_measure_fma_peak(int precision, double* tflops);

/* Total symmetric Dirichlet energy of a triangle parametrisation, for
   callers that cannot allocate device memory (code running while another
   component captures a CUDA graph, hosts whose memory pool forbids outside
   allocations, real-time loops that cannot take an allocation's implicit
   synchronisation).  Inputs and output are the caller's device buffers:
   x_d (2 * n_vertices doubles, interleaved UVs), faces_d (n_faces x 3
   int32), params_d (n_faces x 5 doubles, as TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI),
   f_d (1 double); stream is a cudaStream_t (NULL = default stream).  The
   result equals tad_eval on the same term up to summation-order rounding.
   Allocates nothing: its reduction scratch is a fixed 513 KiB device array
   in the library, so n_faces is limited to 16,777,216 (larger sizes return
   TAD_ERR_ARG).  The first call on each device looks up that array's
   address (make it before any stream capture); every call shares the array,
   so calls that overlap on the GPU race.  No counterpart in the reference:
   TinyAD runs on the CPU and allocates per evaluation. */
TAD_API tad_status tad_eval_symmetric_dirichlet_tri_noalloc(const double* x_d, const int32_t* faces_d,
                                                           const double* params_d, int64_t n_faces,
                                                           double* f_d, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TAD_H */
