/*
 * Kernel instantiations of the small built-in energies: position penalty
 * (N = 1) and the dense quadratic used by the ScalarFunction known-answer
 * tests (N = 1, 2).
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

tad_status launch_builtin_misc(Problem& P, Term& T, const tad_term_eval_args& a)
{
    if (T.energy == TAD_ENERGY_POSITION_PENALTY)
    {
        switch (P.d)
        {
        case 1: return run<1, 1>(a, tad::PositionPenalty<1>{T.vtx_d, T.prm_d});
        case 2: return run<2, 1>(a, tad::PositionPenalty<2>{T.vtx_d, T.prm_d});
        default: return run<3, 1>(a, tad::PositionPenalty<3>{T.vtx_d, T.prm_d});
        }
    }
    // TAD_ENERGY_QUADRATIC
    switch (P.d * 10 + T.N)
    {
    case 11: return run<1, 1>(a, tad::Quadratic<1, 1>{T.vtx_d, T.prm_d});
    case 21: return run<2, 1>(a, tad::Quadratic<2, 1>{T.vtx_d, T.prm_d});
    case 31: return run<3, 1>(a, tad::Quadratic<3, 1>{T.vtx_d, T.prm_d});
    case 12: return run<1, 2>(a, tad::Quadratic<1, 2>{T.vtx_d, T.prm_d});
    default: return run<2, 2>(a, tad::Quadratic<2, 2>{T.vtx_d, T.prm_d});
    }
}

} // namespace tadlib
