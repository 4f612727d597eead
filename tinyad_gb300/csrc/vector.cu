/*
 * Vector functions (include/TinyAD/VectorFunction.hh,
 * Detail/VectorObjectiveTerm.hh) and the Gauss-Newton direction
 * (Utils/GaussNewtonDirection.hh:24-64).
 *
 * A vector problem holds terms whose functors return M residuals per
 * element.  The residuals are numbered term by term, element by element
 * (VectorObjectiveTerm.hh:160-215).  The scalar entry points act on the sum
 * of squares f = sum_i r_i^2: tad_eval is eval_sum_of_squares, the gradient
 * is 2 J^T r, and the Hessian entry points assemble the Gauss-Newton matrix
 * 2 J^T J from the per-element blocks 2 J_e^T J_e through the same pattern,
 * assembly and PCG as scalar problems -- so tad_newton_solve runs
 * Gauss-Newton iterations with the reference's Armijo line search on the
 * sum of squares.  The residual gradients (the Jacobian J, n_outputs x
 * n_vars) and the residual Hessians are evaluated by the same element
 * kernels in the VEC_JACOBIAN / VEC_DERIVATIVES modes and returned in CSR /
 * per-output triplet form.
 */
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "internal.hh"

namespace tadlib {

static tad_status vfail(tad_status s, const char* m) { set_error(m); return s; }

static tad_status ensure_vector(Problem& P)
{
    if (P.kind != 2) return vfail(TAD_ERR_STATE, "not a vector function (no vector terms)");
    return ensure_finalized(P);
}

static tad_status ensure_vec_buffers(Problem& P, int level)
{
    if (level >= 1 && !P.vr) TAD_CUDA_TRY(cudaMalloc(&P.vr, std::max<int64_t>(P.n_outputs_total, 1) * sizeof(double)));
    if (level >= 2 && !P.vJ) TAD_CUDA_TRY(cudaMalloc(&P.vJ, std::max<int64_t>(P.jac_size, 1) * sizeof(double)));
    if (level >= 3 && !P.vHv) TAD_CUDA_TRY(cudaMalloc(&P.vHv, std::max<int64_t>(P.hv_size, 1) * sizeof(double)));
    return TAD_OK;
}

/* Jacobian CSR pattern: row i = output i, columns = the variables of its
   element's used slots, sorted; jmap_h[q] = index of value q in vJ */
static tad_status build_jacobian_pattern(Problem& P, std::vector<int64_t>& jmap)
{
    const int d = P.d;
    P.jptr_h.assign(P.n_outputs_total + 1, 0);
    P.jcol_h.clear();
    jmap.clear();
    std::vector<std::pair<int32_t, int64_t>> row;
    int64_t out = 0;
    for (const Term& T : P.terms)
    {
        const int k = d * T.N;
        for (int64_t e = 0; e < T.n_elem; ++e)
            for (int o = 0; o < T.M; ++o, ++out)
            {
                row.clear();
                for (int a = 0; a < T.N; ++a)
                {
                    const int32_t v = T.rec_h[e * T.N + a];
                    if (v < 0) continue;
                    for (int i = 0; i < d; ++i)
                        row.emplace_back(d * v + i, T.jac_off + (e * T.M + o) * k + a * d + i);
                }
                std::sort(row.begin(), row.end());
                for (const auto& c : row) { P.jcol_h.push_back(c.first); jmap.push_back(c.second); }
                P.jptr_h[out + 1] = (int32_t)P.jcol_h.size();
            }
    }
    if (P.jcol_h.size() >= (size_t(1) << 31)) return vfail(TAD_ERR_ARG, "Jacobian too large for 32-bit indices");
    return TAD_OK;
}

static tad_status jacobian_values(Problem& P, double* J_h)
{
    std::vector<int64_t> jmap;
    tad_status s = build_jacobian_pattern(P, jmap);
    if (s != TAD_OK) return s;
    std::vector<double> vJ(P.jac_size);
    TAD_CUDA_TRY(cudaMemcpyAsync(vJ.data(), P.vJ, P.jac_size * sizeof(double), cudaMemcpyDeviceToHost, P.stream));
    TAD_CUDA_TRY(cudaStreamSynchronize(P.stream));
    for (size_t q = 0; q < jmap.size(); ++q) J_h[q] = vJ[jmap[q]];
    return TAD_OK;
}

/* evaluate the vector terms in `mode`, filling the residual buffers up to `level` */
static tad_status vec_eval(Problem& P, const double* x_h, int mode, int level)
{
    tad_status s = ensure_vector(P);
    if (s != TAD_OK) return s;
    s = ensure_vec_buffers(P, level);
    if (s != TAD_OK) return s;
    TAD_CUDA_TRY(cudaMemcpyAsync(P.x, x_h, P.n_vars * 8, cudaMemcpyHostToDevice, P.stream));
    P.vec_outputs = level;
    s = eval_elements(P, mode, P.x, 0.0, TAD_PREC_FP64);
    P.vec_outputs = 0;
    if (s != TAD_OK) return s;
    return check_device_error(P);
}

} // namespace tadlib

using namespace tadlib;

extern "C" {

TAD_API int64_t tad_n_outputs(const tad_problem* P)
{
    if (!P) return 0;
    int64_t m = 0;
    for (const Term& T : P->terms) m += T.n_elem * T.M;
    return m;
}

TAD_API tad_status tad_vec_eval(tad_problem* P, const double* x_h, double* r_h)
{
    if (!P || !x_h || !r_h) return vfail(TAD_ERR_ARG, "NULL argument");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    tad_status s = vec_eval(*P, x_h, TAD_MODE_VALUE, 1);
    if (s != TAD_OK) return s;
    TAD_CUDA_TRY(cudaMemcpyAsync(r_h, P->vr, P->n_outputs_total * 8, cudaMemcpyDeviceToHost, P->stream));
    TAD_CUDA_TRY(cudaStreamSynchronize(P->stream));
    return TAD_OK;
}

TAD_API tad_status tad_vec_jacobian_nnz(tad_problem* P, int64_t* nnz)
{
    if (!P || !nnz) return vfail(TAD_ERR_ARG, "NULL argument");
    tad_status s = ensure_vector(*P);
    if (s != TAD_OK) return s;
    int64_t n = 0;
    for (const Term& T : P->terms)
        for (int64_t e = 0; e < T.n_elem; ++e)
        {
            int used = 0;
            for (int a = 0; a < T.N; ++a) used += T.rec_h[e * T.N + a] >= 0 ? 1 : 0;
            n += (int64_t)T.M * used * P->d;
        }
    *nnz = n;
    return TAD_OK;
}

TAD_API tad_status tad_vec_jacobian_pattern(tad_problem* P, int32_t* outer, int32_t* inner)
{
    if (!P || !outer || !inner) return vfail(TAD_ERR_ARG, "NULL argument");
    tad_status s = ensure_vector(*P);
    if (s != TAD_OK) return s;
    std::vector<int64_t> jmap;
    s = build_jacobian_pattern(*P, jmap);
    if (s != TAD_OK) return s;
    std::copy(P->jptr_h.begin(), P->jptr_h.end(), outer);
    std::copy(P->jcol_h.begin(), P->jcol_h.end(), inner);
    return TAD_OK;
}

TAD_API tad_status tad_vec_eval_with_jacobian(tad_problem* P, const double* x_h, double* r_h, double* J_values_h)
{
    if (!P || !x_h || !r_h || !J_values_h) return vfail(TAD_ERR_ARG, "NULL argument");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    tad_status s = vec_eval(*P, x_h, TAD_MODE_VEC_JACOBIAN, 2);
    if (s != TAD_OK) return s;
    TAD_CUDA_TRY(cudaMemcpyAsync(r_h, P->vr, P->n_outputs_total * 8, cudaMemcpyDeviceToHost, P->stream));
    return jacobian_values(*P, J_values_h);
}

TAD_API tad_status tad_vec_hessians_nnz(tad_problem* P, int64_t* nnz)
{
    if (!P || !nnz) return vfail(TAD_ERR_ARG, "NULL argument");
    tad_status s = ensure_vector(*P);
    if (s != TAD_OK) return s;
    int64_t n = 0;
    for (const Term& T : P->terms)
        for (int64_t e = 0; e < T.n_elem; ++e)
        {
            int used = 0;
            for (int a = 0; a < T.N; ++a) used += T.rec_h[e * T.N + a] >= 0 ? 1 : 0;
            n += (int64_t)T.M * (used * P->d) * (used * P->d);
        }
    *nnz = n;
    return TAD_OK;
}

/* r, J and the residual Hessians: output i owns triplets
   [H_ptr[i], H_ptr[i+1]) of (H_row, H_col, H_val), the full k_used x k_used
   block over its element's variables in local order (row by row), as the
   reference emits them (VectorObjectiveTerm.hh:283-294). */
TAD_API tad_status tad_vec_eval_with_derivatives(tad_problem* P, const double* x_h, double* r_h, double* J_values_h,
                                                 int64_t* H_ptr, int32_t* H_row, int32_t* H_col, double* H_val)
{
    if (!P || !x_h || !r_h || !J_values_h || !H_ptr || !H_row || !H_col || !H_val)
        return vfail(TAD_ERR_ARG, "NULL argument");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    tad_status s = vec_eval(*P, x_h, TAD_MODE_VEC_DERIVATIVES, 3);
    if (s != TAD_OK) return s;
    TAD_CUDA_TRY(cudaMemcpyAsync(r_h, P->vr, P->n_outputs_total * 8, cudaMemcpyDeviceToHost, P->stream));
    std::vector<double> hv(P->hv_size);
    TAD_CUDA_TRY(cudaMemcpyAsync(hv.data(), P->vHv, P->hv_size * 8, cudaMemcpyDeviceToHost, P->stream));
    s = jacobian_values(*P, J_values_h);   // synchronises the stream
    if (s != TAD_OK) return s;
    const int d = P->d;
    int64_t out = 0, q = 0;
    H_ptr[0] = 0;
    std::vector<int32_t> gi;
    for (const Term& T : P->terms)
    {
        const int k = d * T.N, nh = k * (k + 1) / 2;
        for (int64_t e = 0; e < T.n_elem; ++e)
        {
            gi.clear();
            std::vector<int> li;
            for (int a = 0; a < T.N; ++a)
            {
                const int32_t v = T.rec_h[e * T.N + a];
                if (v < 0) continue;
                for (int c = 0; c < d; ++c) { gi.push_back(d * v + c); li.push_back(a * d + c); }
            }
            for (int o = 0; o < T.M; ++o, ++out)
            {
                const double* hp = hv.data() + T.hv_off + (e * T.M + o) * nh;
                for (size_t i = 0; i < gi.size(); ++i)
                    for (size_t j = 0; j < gi.size(); ++j, ++q)
                    {
                        const int a = li[i], b = li[j];
                        H_row[q] = gi[i];
                        H_col[q] = gi[j];
                        H_val[q] = a <= b ? hp[a * k - (a * (a - 1)) / 2 + (b - a)] : hp[b * k - (b * (b - 1)) / 2 + (a - b)];
                    }
                H_ptr[out + 1] = q;
            }
        }
    }
    return TAD_OK;
}

/* f = |r|^2, g = 2 J^T r, r and J (VectorFunctionImpl.hh:271-283) */
TAD_API tad_status tad_eval_sum_of_squares_with_derivatives(tad_problem* P, const double* x_h, double* f, double* g_h,
                                                            double* r_h, double* J_values_h)
{
    if (!P || !x_h || !f || !g_h || !r_h || !J_values_h) return vfail(TAD_ERR_ARG, "NULL argument");
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    tad_status s = vec_eval(*P, x_h, TAD_MODE_VEC_JACOBIAN, 2);
    if (s != TAD_OK) return s;
    s = assemble(*P, true, false, TAD_PREC_FP64);
    if (s != TAD_OK) return s;
    TAD_CUDA_TRY(cudaMemcpyAsync(r_h, P->vr, P->n_outputs_total * 8, cudaMemcpyDeviceToHost, P->stream));
    TAD_CUDA_TRY(cudaMemcpyAsync(g_h, P->g, P->n_vars * 8, cudaMemcpyDeviceToHost, P->stream));
    TAD_CUDA_TRY(cudaMemcpyAsync(P->hs, P->ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, P->stream));
    s = jacobian_values(*P, J_values_h);
    if (s != TAD_OK) return s;
    *f = P->hs->f;
    return TAD_OK;
}

/* gauss_newton_direction(r, J, solver, w) (GaussNewtonDirection.hh:24-47):
   d = -(J^T J + w I)^-1 J^T r at x, solved as (2 J^T J + 2 w I) d = -2 J^T r
   with the assembled Gauss-Newton matrix and the device PCG. */
TAD_API tad_status tad_gauss_newton_direction(tad_problem* P, const double* x_h, double w, double* d_h, double* f,
                                              double* g_h)
{
    if (!P || !x_h || !d_h) return vfail(TAD_ERR_ARG, "NULL argument");
    if (P->kind != 2) return vfail(TAD_ERR_STATE, "not a vector function (no vector terms)");
    return tad_newton_direction(P, x_h, 0, 0.0, 2.0 * w, d_h, f, g_h);
}

} // extern "C"
