"""GPU parity at sizes where the solver works as it does on the benchmark
meshes: a 256^2-grid disk (about 103k faces) and a 12^3 tetrahedral cube
with the twist penalties (10,368 tets).  On these, the late Newton steps need
hundreds of block-Jacobi PCG iterations, so the smoothed-aggregation V-cycle
takes over, in FP64 and in FP32 (mixed precision).

Checked against the oracle (the CPU restatement of TinyAD's path, sparse
LDL^T Newton, tests/NewtonTest.cc:69-95 and Utils/NewtonDirection.hh:25-48):
  * FP64 f, g and the projected H within 1e-10 normwise relative error, at
    the initial state and at the state after a few device Newton iterations;
  * mixed precision f within 1e-11, g within 1e-9, H within 5e-5 (double-
    float values and gradients, FP32 Hessian arithmetic), at the same states
    -- looser than the 6.4k-face tests' 1e-12 / 1e-10: the per-element
    double-float errors (about 4e-14 relative) add up over 16x more faces,
    and near equilibrium the summed gradient is small against its terms;
  * the final energy of a device solve (the benchmark's policy: PCG to a 1e-2
    relative residual) within 1e-8 of the oracle's converged energy, for FP64
    and mixed precision.
"""
import numpy as np
import pytest

from conftest import rel_err, sparse_rel_err
from tinyad_gb300 import meshes

pytestmark = pytest.mark.gpu

TOL = 1e-10
BENCH_POLICY = dict(pcg_rel_tol=1e-2, pcg_max_iters=2000, forcing=0, refine_max_iters=3, refine_rel_tol=1e-8)


def _oracle_converged(p, x0, max_iters=40):
    """The oracle's Newton loop, one iteration at a time, until the energy
    stops changing (relative 1e-15) or max_iters."""
    x = x0.copy()
    f_prev = None
    for _ in range(max_iters):
        x, fh, _ = p.newton(x, 1)
        if f_prev is not None and abs(fh[-1] - f_prev) <= 1e-15 * abs(fh[-1]):
            break
        f_prev = fh[-1]
    return x, float(fh[-1])


def _device_states(tad, w, prec, iters):
    """x after `iters` device Newton iterations with the benchmark's policy."""
    fn = tad.ScalarFunction.from_workload(w, precision=prec, **BENCH_POLICY)
    x, fh = fn.newton_solve(w.x0, iters)
    return x


def _eval_checks(tad, oracle_p, w, xs):
    f64 = tad.ScalarFunction.from_workload(w, precision=tad.PREC_FP64)
    fmx = tad.ScalarFunction.from_workload(w, precision=tad.PREC_MIXED)
    for x in xs:
        fo, go, Ho = oracle_p.eval_with_hessian_proj(x)
        f, g, H = f64.eval_with_hessian_proj(x)
        assert rel_err(f, fo) <= TOL and rel_err(g, go) <= TOL, (rel_err(f, fo), rel_err(g, go))
        assert H.nnz == Ho.nnz and sparse_rel_err(H, Ho) <= TOL, sparse_rel_err(H, Ho)
        f, g, H = fmx.eval_with_hessian_proj(x)
        assert rel_err(f, fo) <= 1e-11 and rel_err(g, go) <= 1e-9, (rel_err(f, fo), rel_err(g, go))
        assert sparse_rel_err(H, Ho) <= 5e-5, sparse_rel_err(H, Ho)


def _final_energy_checks(tad, w, f_star, iters):
    for prec in (tad.PREC_FP64, tad.PREC_MIXED):
        fn = tad.ScalarFunction.from_workload(w, precision=prec, **BENCH_POLICY)
        x, fh = fn.newton_solve(w.x0, iters)
        assert abs(fh[-1] - f_star) <= 1e-8 * abs(f_star), (prec, fh[-4:], f_star)
        assert abs(fn.eval(x) - fh[-1]) <= 1e-12 * abs(fh[-1])


@pytest.fixture(scope="module")
def disk256(oracle):
    w = meshes.disk_param(256, seed=2)
    p = oracle.Problem.from_workload(w)
    return w, p


@pytest.fixture(scope="module")
def tet12(oracle):
    w = meshes.tet_twist(12, seed=1)
    p = oracle.Problem.from_workload(w)
    return w, p


def test_disk256_eval_parity(tad, disk256):
    w, p = disk256
    assert w.n_elements > 100_000
    _eval_checks(tad, p, w, [w.x0, _device_states(tad, w, tad.PREC_FP64, 8)])


def test_disk256_newton_final_energy(tad, disk256):
    w, p = disk256
    _, f_star = _oracle_converged(p, w.x0)
    _final_energy_checks(tad, w, f_star, 40)


def test_disk256_late_steps_use_the_vcycle(tad, disk256):
    """A late Newton step of the large disk that block Jacobi alone needs more
    than 60 PCG iterations for finishes under the V-cycle in a third of them
    or fewer (FP64 and FP32), and meets the solve's relative tolerance."""
    w, _ = disk256
    stepper = tad.ScalarFunction.from_workload(w, precision=tad.PREC_FP64, **BENCH_POLICY)
    bj = {p: tad.ScalarFunction.from_workload(w, precision=p, preconditioner=0, **BENCH_POLICY)
          for p in (tad.PREC_FP64, tad.PREC_MIXED)}
    x = w.x0.copy()
    for _ in range(30):
        bj[tad.PREC_FP64].newton_direction(x)
        if bj[tad.PREC_FP64].last_solve_stats()["pcg_iters"] > 60:
            break
        x, _ = stepper.newton_solve(x, 1)
    else:
        pytest.fail("no Newton state needed more than 60 block-Jacobi iterations")
    for prec, tol in ((tad.PREC_FP64, 1.001e-2), (tad.PREC_MIXED, 1.5e-2)):
        bj[prec].newton_direction(x)
        it_bj = bj[prec].last_solve_stats()["pcg_iters"]
        fn = tad.ScalarFunction.from_workload(w, precision=prec, preconditioner=1, **BENCH_POLICY)
        d, _, g = fn.newton_direction(x)
        it_amg = fn.last_solve_stats()["pcg_iters"]
        _, _, H = fn.eval_with_hessian_proj(x)
        assert np.linalg.norm(H @ d + g) <= tol * np.linalg.norm(g)
        assert it_bj > 3 * it_amg, (prec, it_bj, it_amg)


def test_tet12_eval_parity(tad, tet12):
    w, p = tet12
    _eval_checks(tad, p, w, [w.x0, _device_states(tad, w, tad.PREC_FP64, 3)])


def test_tet12_newton_final_energy(tad, tet12):
    w, p = tet12
    _, f_star = _oracle_converged(p, w.x0)
    _final_energy_checks(tad, w, f_star, 40)
