/*
 * Adjoint of the Projected-Newton solution with respect to the rest shape.
 *
 * For x*(P) = argmin_x E(x, P), a loss L(x*) has
 *   dL/dP = -(d2E/dx dP)^T lambda,   H lambda = dL/dx,
 * with H the (optionally PSD-projected) Hessian at x*.  The linear solve is
 * the library's PCG; the mixed blocks d2E_e/dx_e dP_e (6 x 9 per triangle)
 * are recomputed per element by forward mode with a block-restricted
 * Hessian (tad::MixedScalar<6, 9>, the reference's truncated-Hessian scalar
 * Scalar<15, double, true, 0, 6, 6, 9>, include/TinyAD/Scalar.hh:24,
 * :186-196) -- element Hessians are not stored.  Each element writes
 * -B_e^T lambda_e into its three vertex slots; the per-vertex sum is the same
 * element-ordered gather as the gradient assembly (deterministic).
 *
 * Rest positions enter through the built-in symmetric Dirichlet triangle
 * energy (tad::symmetric_dirichlet_tri_rest); other terms (position
 * penalties) do not depend on them.
 */
#include "internal.hh"
#include "../../include/tad/Energies.cuh"

namespace tadlib {

__global__ void __launch_bounds__(128) k_adjoint_tri(int64_t n_elem, const int32_t* __restrict__ vtx,
                                                     const double* __restrict__ x, const double* __restrict__ rest,
                                                     const double* __restrict__ lambda, double* __restrict__ out)
{
    using M = tad::MixedScalar<6, 9, double>;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n_elem) return;
    int v[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) v[a] = vtx[e * 3 + a];
    tad::Vec<M, 2> u[3];
    tad::Vec<M, 3> P[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
#pragma unroll
        for (int i = 0; i < 2; ++i) u[a][i] = M(x[2 * (int64_t)v[a] + i], 2 * a + i);
#pragma unroll
        for (int i = 0; i < 3; ++i) P[a][i] = M(rest[3 * (int64_t)v[a] + i], 6 + 3 * a + i);
    }
    const M E = tad::symmetric_dirichlet_tri_rest(u[0], u[1], u[2], P[0], P[1], P[2]);
    double lam[6];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int i = 0; i < 2; ++i) lam[2 * a + i] = lambda[2 * (int64_t)v[a] + i];
    const bool finite = isfinite(E.val);
#pragma unroll
    for (int j = 0; j < 9; ++j)
    {
        double c = 0.0;
#pragma unroll
        for (int i = 0; i < 6; ++i) c -= E.blk[i * 9 + j] * lam[i];
        out[e * 9 + j] = finite ? c : 0.0;
    }
}

/* out3[v] = sum over v's element slots of buf[slot][3], in element order */
__global__ void k_gather3(int64_t nh, const int32_t* __restrict__ gptr, const int32_t* __restrict__ gidx,
                          const double* __restrict__ buf, double* __restrict__ out)
{
    const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (u >= nh) return;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int32_t q = gptr[u]; q < gptr[u + 1]; ++q)
    {
        const int64_t s = gidx[q];
#pragma unroll
        for (int i = 0; i < 3; ++i) acc[i] += buf[s * 3 + i];
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) out[u * 3 + i] = acc[i];
}

} // namespace tadlib

using namespace tadlib;

extern "C" TAD_API tad_status tad_adjoint_rest_gradient(tad_problem* P, const double* x_h, const double* dLdx_h,
                                                        const double* rest_h, int projected, double proj_eps,
                                                        double* dLdrest_h, double* lambda_h, int* pcg_iters)
{
    if (!P || !x_h || !dLdx_h || !rest_h || !dLdrest_h) { set_error("NULL argument"); return TAD_ERR_ARG; }
    if (P->d != 2) { set_error("the rest-shape adjoint needs var_dim 2 (triangle parametrisation)"); return TAD_ERR_ARG; }
    TAD_CUDA_TRY(cudaSetDevice(P->device));
    tad_status s = ensure_finalized(*P);
    if (s != TAD_OK) return s;
    Problem& Q = *P;
    cudaStream_t st = Q.stream;
    const int64_t n = Q.n_vars, nh = Q.n_handles;
    TAD_CUDA_TRY(cudaMemcpyAsync(Q.x, x_h, n * 8, cudaMemcpyHostToDevice, st));
    TAD_CUDA_TRY(cudaMemcpyAsync(Q.rhs, dLdx_h, n * 8, cudaMemcpyHostToDevice, st));
    s = eval_full(Q, Q.x, projected ? TAD_MODE_HESSIAN_PROJ : TAD_MODE_HESSIAN, proj_eps, TAD_PREC_FP64);
    if (s != TAD_OK) return s;
    s = check_device_error(Q);
    if (s != TAD_OK) return s;
    int it = 0;
    tad_status ps = pcg_solve(Q, Q.rhs, Q.dx, 0.0, TAD_PREC_FP64, Q.settings.pcg_rel_tol, Q.settings.pcg_max_iters, &it);
    if (ps != TAD_OK && ps != TAD_ERR_PCG_NOCONV) return ps;
    if (pcg_iters) *pcg_iters = it;
    double *rest_d = nullptr, *buf = nullptr, *out_d = nullptr;
    TAD_CUDA_TRY(cudaMalloc(&rest_d, nh * 3 * 8));
    TAD_CUDA_TRY(cudaMalloc(&buf, std::max<int64_t>(Q.n_slots_total, 1) * 3 * 8));
    TAD_CUDA_TRY(cudaMalloc(&out_d, nh * 3 * 8));
    TAD_CUDA_TRY(cudaMemcpyAsync(rest_d, rest_h, nh * 3 * 8, cudaMemcpyHostToDevice, st));
    TAD_CUDA_TRY(cudaMemsetAsync(buf, 0, std::max<int64_t>(Q.n_slots_total, 1) * 3 * 8, st));
    for (Term& T : Q.terms)
    {
        if (T.energy != TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI || T.n_elem == 0) continue;
        k_adjoint_tri<<<(unsigned)((T.n_elem + 127) / 128), 128, 0, st>>>(T.n_elem, T.vtx_d, Q.x, rest_d, Q.dx,
                                                                         buf + T.slot_off * 3);
        Q.n_launches += 1;
    }
    k_gather3<<<(unsigned)((nh + 255) / 256), 256, 0, st>>>(nh, Q.gptr, Q.gidx, buf, out_d);
    Q.n_launches += 1;
    TAD_CUDA_TRY(cudaMemcpyAsync(dLdrest_h, out_d, nh * 3 * 8, cudaMemcpyDeviceToHost, st));
    if (lambda_h) TAD_CUDA_TRY(cudaMemcpyAsync(lambda_h, Q.dx, n * 8, cudaMemcpyDeviceToHost, st));
    TAD_CUDA_TRY(cudaStreamSynchronize(st));
    cudaFree(rest_d);
    cudaFree(buf);
    cudaFree(out_d);
    TAD_CUDA_TRY(cudaGetLastError());
    if (ps == TAD_ERR_PCG_NOCONV) set_error("adjoint linear solve did not reach its tolerance");
    return ps;
}
