/* Second-order kernel of the built-in tet energy (k = 12), mixed. */
#include "internal.hh"
#include "../../include/tad/ElementKernels.cuh"
#include "../../include/tad/Energies.cuh"

namespace tadlib {

void tet_hessian_mixed(const tad::ElemLaunch& L, const tad::SymmetricDirichletTet& e, cudaStream_t s)
{
    tad::launch_elements_hessian<3, 4, float>(L, e, s);
}

} // namespace tadlib
