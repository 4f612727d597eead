/*
 * Kernel instantiations of the built-in residual functors of vector terms
 * (tad_vector_energy): the symmetric Dirichlet residuals of a triangle
 * (d = 2, N = 3, 8 outputs) and position residuals (N = 1, d outputs).
 */
#include "internal.hh"
#include "../../include/tad/ElementKernels.cuh"
#include "../../include/tad/Energies.cuh"

namespace tadlib {

template <int d, int N, int M, typename E>
static tad_status run(const tad_term_eval_args& a, const E& energy)
{
    tad::launch_vector_elements<d, N, M>(a.mode, a.precision, tad::make_launch(a), energy, (cudaStream_t)a.stream);
    return TAD_OK;
}

tad_status launch_builtin_vec(Problem& P, Term& T, const tad_term_eval_args& a)
{
    if (T.energy == TAD_VEC_SYMMETRIC_DIRICHLET_TRI)
        return run<2, 3, 8>(a, tad::SymmetricDirichletTriResiduals{T.vtx_d, T.prm_d});
    switch (P.d)
    {
    case 1: return run<1, 1, 1>(a, tad::PositionResiduals<1>{T.vtx_d, T.prm_d});
    case 2: return run<2, 1, 2>(a, tad::PositionResiduals<2>{T.vtx_d, T.prm_d});
    default: return run<3, 1, 3>(a, tad::PositionResiduals<3>{T.vtx_d, T.prm_d});
    }
}

} // namespace tadlib
