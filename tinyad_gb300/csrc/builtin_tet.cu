/*
 * Kernel instantiations of the built-in tet energy (d = 3 symmetric
 * Dirichlet, k = 12): first-order modes here; the two second-order kernels
 * (FP64 and mixed) are in builtin_tet_h64.cu / builtin_tet_h32.cu so the
 * three large translation units compile in parallel.
 */
#include "internal.hh"
#include "../../include/tad/ElementKernels.cuh"
#include "../../include/tad/Energies.cuh"

namespace tadlib {

void tet_hessian_fp64(const tad::ElemLaunch& L, const tad::SymmetricDirichletTet& e, cudaStream_t s);
void tet_hessian_mixed(const tad::ElemLaunch& L, const tad::SymmetricDirichletTet& e, cudaStream_t s);

tad_status launch_builtin_tet(Problem& P, Term& T, const tad_term_eval_args& a)
{
    (void)P;
    const tad::ElemLaunch L = tad::make_launch(a);
    const tad::SymmetricDirichletTet energy{T.vtx_d, T.prm_d};
    const cudaStream_t s = (cudaStream_t)a.stream;
    if (a.mode == TAD_MODE_HESSIAN || a.mode == TAD_MODE_HESSIAN_PROJ)
    {
        if (a.precision == TAD_PREC_MIXED) tet_hessian_mixed(L, energy, s);
        else tet_hessian_fp64(L, energy, s);
    }
    else tad::launch_elements_first_order<3, 4>(a.mode, L, energy, s, a.precision);
    return TAD_OK;
}

} // namespace tadlib
