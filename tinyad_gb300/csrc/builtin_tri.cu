/*
 * Kernel instantiations of the built-in triangle energies (d = 2 symmetric
 * Dirichlet, k = 6; Dirichlet/Laplacian for d = 1..3).
 */
#include "internal.hh"
#include "../../include/tad/ElementKernels.cuh"
#include "../../include/tad/Energies.cuh"

namespace tadlib {

template <int d, int N, typename E>
static tad_status run(const tad_term_eval_args& a, const E& energy)
{
    tad::launch_elements<d, N>(a.mode, a.precision, tad::make_launch(a), energy, (cudaStream_t)a.stream);
    return TAD_OK;
}

tad_status launch_builtin_tri(Problem& P, Term& T, const tad_term_eval_args& a)
{
    if (T.energy == TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI)
        return run<2, 3>(a, tad::SymmetricDirichletTri{T.vtx_d, T.prm_d});
    switch (P.d)
    {
    case 1: return run<1, 3>(a, tad::DirichletTri<1>{T.vtx_d, T.prm_d});
    case 2: return run<2, 3>(a, tad::DirichletTri<2>{T.vtx_d, T.prm_d});
    default: return run<3, 3>(a, tad::DirichletTri<3>{T.vtx_d, T.prm_d});
    }
}

} // namespace tadlib
