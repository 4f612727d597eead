"""VectorFunction and Gauss-Newton on the device (include/TinyAD/VectorFunction.hh,
Utils/GaussNewtonDirection.hh), pinned to tests/GaussNewtonTest.cc: the
residual form of the symmetric Dirichlet + position penalty problem has the
scalar problem's energy and gradient (checked against the oracle), J matches
finite differences of r, the residual Hessians satisfy
Hess f = sum_i 2 (r_i Hess r_i + grad r_i grad r_i^T) against the oracle's
exact Hessian, the Gauss-Newton direction matches a direct solve, and the
reference's Gauss-Newton loop reaches f = 4 on the planar test mesh."""
import numpy as np
import pytest

from conftest import rel_err
from tinyad_gb300 import meshes

pytestmark = pytest.mark.gpu


def _vector_function(tad, w, **kw):
    vf = tad.VectorFunction(w.var_dim, w.n_handles, **kw)
    for energy, handles, params, m in meshes.residual_terms(w):
        vf.add_elements(energy, handles, params, m)
    return vf


def test_sum_of_squares_matches_scalar_energy(tad, oracle):
    w = meshes.disk_param(16, seed=7)
    vf = _vector_function(tad, w)
    p = oracle.Problem.from_workload(w)
    x = w.x0
    fo, go, _ = p.eval_with_hessian_proj(x)
    assert vf.n_outputs == 8 * w.terms[0].handles.shape[0]
    assert rel_err(vf.eval_sum_of_squares(x), fo) <= 1e-12
    r = vf.eval_vector(x)
    assert rel_err(float(r @ r), fo) <= 1e-12
    f, g, r2, J = vf.eval_sum_of_squares_with_derivatives(x)
    assert rel_err(f, fo) <= 1e-12 and rel_err(g, go) <= 1e-11
    assert np.array_equal(r, r2)
    assert rel_err(2.0 * (J.T @ r2), g) <= 1e-13
    fg, gg = vf.eval_with_gradient(x)
    assert rel_err(fg, fo) <= 1e-12 and rel_err(gg, go) <= 1e-11


def test_jacobian_and_residual_hessians(tad, oracle):
    w = meshes.disk_param(10, seed=8)
    vf = _vector_function(tad, w)
    x = w.x0
    r, J = vf.eval_with_jacobian(x)
    # J by central differences of r
    rng = np.random.default_rng(2)
    for _ in range(4):
        v = rng.standard_normal(w.n_vars)
        v /= np.linalg.norm(v)
        h = 1e-6
        fd = (vf.eval_vector(x + h * v) - vf.eval_vector(x - h * v)) / (2 * h)
        assert rel_err(J @ v, fd) <= 1e-6
    # Hess f = sum_i 2 (r_i Hess r_i + grad r_i grad r_i^T), against the oracle's exact Hessian
    r3, J3, Hs = vf.eval_with_derivatives(x)
    assert np.array_equal(r, r3) and rel_err(J3.toarray(), J.toarray()) == 0.0
    assert len(Hs) == vf.n_outputs
    H = 2.0 * (J.T @ J).toarray()
    for i, Hi in enumerate(Hs):
        H += 2.0 * r[i] * Hi.toarray()
    p = oracle.Problem.from_workload(w)
    _, _, Ho = p.eval_with_derivatives(x)
    assert rel_err(H, Ho.toarray()) <= 1e-10


@pytest.mark.parametrize("w_identity", [1e-12, 0.1])
def test_gauss_newton_direction(tad, w_identity):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    w = meshes.disk_param(16, seed=9)
    vf = _vector_function(tad, w, pcg_rel_tol=1e-12, pcg_max_iters=5000)
    x = w.x0
    f, g, r, J = vf.eval_sum_of_squares_with_derivatives(x)
    d, fd_, gd = vf.gauss_newton_direction(x, w_identity)
    A = (J.T @ J + w_identity * sp.identity(w.n_vars)).tocsc()
    rhs = -(J.T @ r)
    # the rigid translations of the parametrisation are a null space of J^T J:
    # with w = 1e-12 the direction is pinned by the residual of the system, with
    # w = 0.1 also by a direct solve
    assert rel_err(A @ d, rhs) <= 1e-8
    if w_identity > 1e-9:
        assert rel_err(d, spla.spsolve(A, rhs)) <= 1e-8
    assert rel_err(fd_, f) == 0.0 and rel_err(gd, g) <= 1e-13


def test_gauss_newton_planar(tad, oracle):
    """tests/GaussNewtonTest.cc: 20 Gauss-Newton steps (w = 1e-12) with the
    Armijo line search on the sum of squares; at every step f and g equal the
    scalar formulation's; the loop ends at f = 4 with g = 0 (to 0.1)."""
    w = meshes.planar_test_mesh()
    vf = _vector_function(tad, w, pcg_rel_tol=1e-12, pcg_max_iters=1000)
    p = oracle.Problem.from_workload(w)
    x = w.x0.copy()
    for _ in range(20):
        fo, go, _ = p.eval_with_hessian_proj(x)
        f, g, r, J = vf.eval_sum_of_squares_with_derivatives(x)
        assert abs(f - fo) <= 1e-12 * max(1.0, abs(fo))
        assert np.max(np.abs(g - go)) <= 1e-12 * max(1.0, np.max(np.abs(go)))
        d, _, _ = vf.gauss_newton_direction(x, 1e-12)
        x = vf.line_search(x, d, f, g)
    f, g, _, _ = vf.eval_sum_of_squares_with_derivatives(x)
    assert abs(f - 4.0) <= 0.1 and np.max(np.abs(g)) <= 0.1
    # the fused device loop runs the same Gauss-Newton iterations
    x2, fh = vf.newton_solve(w.x0.copy(), 20)
    assert abs(fh[-1] - 4.0) <= 0.1
    assert np.all(np.diff(fh) <= 1e-12 * abs(fh[0]))


def test_vector_and_scalar_terms_do_not_mix(tad):
    vf = tad.VectorFunction(2, 3)
    vf.add_elements(meshes.TAD_VEC_POSITION, [[0]], [[1.0, 2.0, 1.0]], 2)
    with pytest.raises(tad.TinyADError):
        tad.ScalarFunction.add_elements(vf, meshes.TAD_ENERGY_POSITION_PENALTY, [[1]], [[0.0, 0.0, 1.0]])
