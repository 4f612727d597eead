/*
 * Kernel instantiations of the built-in tet energy (d = 3 symmetric
 * Dirichlet, k = 12).
 */
#include "internal.hh"
#include "../../include/tad/ElementKernels.cuh"
#include "../../include/tad/Energies.cuh"

namespace tadlib {

tad_status launch_builtin_tet(Problem& P, Term& T, const tad_term_eval_args& a)
{
    (void)P;
    tad::launch_elements<3, 4>(a.mode, a.precision, tad::make_launch(a),
                               tad::SymmetricDirichletTet{T.vtx_d, T.prm_d}, (cudaStream_t)a.stream);
    return TAD_OK;
}

} // namespace tadlib
