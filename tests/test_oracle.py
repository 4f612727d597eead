"""CPU tests: pin the oracle (the CPU restatement of TinyAD's path) against
the reference's own known answers and tests (see each test's citation)."""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import rel_err, sparse_rel_err, torus_mesh
from tinyad_gb300 import meshes

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")


def _scalar_op(oracle, op, a, b):
    L = oracle.lib()
    out = np.zeros(3)
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    dp = ctypes.POINTER(ctypes.c_double)
    rc = L.oracle_scalar_op(op, a.ctypes.data_as(dp), b.ctypes.data_as(dp), out.ctypes.data_as(dp))
    assert rc == 0
    return out


def test_known_answers(oracle):
    """Operator known answers of tests/ScalarTest{Unary,Binary}Operators.cc."""
    cases = json.load(open(GOLDEN))
    assert len(cases) >= 30
    for c in cases:
        got = _scalar_op(oracle, c["op"], c["a"], c["b"])
        np.testing.assert_allclose(got, c["expected"], rtol=0, atol=c["tol"] * max(1.0, np.max(np.abs(c["expected"]))),
                                   err_msg=f'{c["name"]} ({c["source"]})')


def test_hessian_block(oracle):
    """Truncated Hessian blocks equal the full Hessian's blocks
    (tests/ScalarTestHessianBlock.cc:50-100)."""
    L = oracle.lib()
    dp = ctypes.POINTER(ctypes.c_double)
    x = np.array([10.0, 1.0, 15.0, 3.0, 2.0, 2.0])
    xr = np.array([1.0, 1.0, 2.0, 1.0, 1.0, 2.0])
    for which in range(5):
        full = np.zeros(36)
        blk = np.zeros(36)
        assert L.oracle_symdir_hessian_block(which, x.ctypes.data_as(dp), xr.ctypes.data_as(dp),
                                             full.ctypes.data_as(dp), blk.ctypes.data_as(dp)) == 0
        assert np.max(np.abs(full - blk)) <= 1e-16 * max(1.0, np.max(np.abs(full)))
        assert np.all(np.isfinite(full))


def _quad_params(A, b, c):
    A = np.asarray(A, np.float64)
    return np.concatenate([A.ravel(), np.asarray(b, np.float64), [c]])[None, :]


def test_scalar_function_quadratics(oracle):
    """tests/ScalarFunctionTest.cc:46-151 (1D, 2D, non-convex)."""
    # 1D: 2 x^2 + x + 1 at x = 1
    p = oracle.Problem(1, 1)
    p.add_elements(meshes.TAD_ENERGY_QUADRATIC, np.array([[0]]), _quad_params([[2.0]], [1.0], 1.0))
    f, g, H = p.eval_with_hessian_proj(np.array([1.0]))
    assert abs(f - 4.0) <= 1e-16 and abs(g[0] - 5.0) <= 1e-16 and abs(H[0, 0] - 4.0) <= 1e-16
    # 2D: 2x^2 + 2xy + y^2 + x + 1 at (1, 2)
    A2 = [[2.0, 1.0], [1.0, 1.0]]
    p = oracle.Problem(2, 1)
    p.add_elements(meshes.TAD_ENERGY_QUADRATIC, np.array([[0]]), _quad_params(A2, [1.0, 0.0], 1.0))
    x = np.array([1.0, 2.0])
    for f, g, H in (p.eval_with_derivatives(x), p.eval_with_hessian_proj(x)):
        assert f == 12.0 and list(g) == [9.0, 6.0]
        assert np.array_equal(H.toarray(), [[4.0, 2.0], [2.0, 2.0]])
    # non-convex: the negation; projected Hessian is positive definite
    p = oracle.Problem(2, 1)
    p.add_elements(meshes.TAD_ENERGY_QUADRATIC, np.array([[0]]),
                   _quad_params(-np.array(A2), [-1.0, 0.0], -1.0))
    f, g, H = p.eval_with_derivatives(x)
    assert f == -12.0 and list(g) == [-9.0, -6.0]
    assert np.array_equal(H.toarray(), [[-4.0, -2.0], [-2.0, -2.0]])
    f, g, Hp = p.eval_with_hessian_proj(x)
    assert np.all(np.linalg.eigvalsh(Hp.toarray()) > 0)


def test_planar_newton(oracle):
    """tests/NewtonTest.cc:12-111: nnz = 4V + 8(V+F-1); f -> 4, g -> 0 within
    1e-15 after 10 Projected-Newton iterations; deterministic."""
    w = meshes.planar_test_mesh()
    p = oracle.Problem.from_workload(w)
    f, g, H = p.eval_with_hessian_proj(w.x0)
    assert H.nnz == 4 * 6 + 8 * (6 + 4 - 1)
    x1, fh1, _ = p.newton(w.x0, 10)
    x2, fh2, _ = oracle.Problem.from_workload(w).newton(w.x0, 10)
    f, g, H = p.eval_with_hessian_proj(x1)
    assert abs(p.eval(x1) - f) <= 1e-15
    assert abs(f - 4.0) <= 1e-15
    assert np.max(np.abs(g)) <= 1e-15
    assert np.array_equal(x1, x2) and np.array_equal(fh1, fh2)


def test_laplacian(oracle):
    """Hessian of the Dirichlet energy 1/4 sum |b-a|^2 + ... equals the graph
    Laplacian with the same nnz (tests/DynamicElementsTest.cc:60-91)."""
    import scipy.sparse as sp
    nv, F = torus_mesh()
    p = oracle.Problem(1, nv)
    p.add_elements(meshes.TAD_ENERGY_DIRICHLET_TRI, F, np.full((F.shape[0], 1), 0.25))
    f, g, H = p.eval_with_derivatives(np.zeros(nv))
    rows, cols, vals = [], [], []
    for t in F:
        for i in range(3):
            v1, v2 = t[i], t[(i + 1) % 3]
            rows += [v1, v1]
            cols += [v1, v2]
            vals += [1.0, -1.0]
    Lref = sp.coo_matrix((vals, (rows, cols)), shape=(nv, nv)).tocsc()
    Lref.sum_duplicates()
    assert H.nnz == Lref.nnz
    assert abs(H - Lref).max() <= 1e-12


def test_projection_matches_eigh(oracle):
    """Projected element Hessians = eigenvalue clamp of the unprojected ones
    (HessianProjection.hh:48-101), checked against numpy's eigh."""
    rng = np.random.default_rng(3)
    for trial in range(20):
        w = meshes.planar_test_mesh()
        t = w.terms[0]
        e = trial % 4
        p = oracle.Problem(2, 6)
        p.add_elements(t.energy, t.handles[e:e + 1], t.params[e:e + 1])
        x = w.x0 + rng.normal(scale=0.05, size=w.x0.size)
        f, g, H = p.eval_with_derivatives(x)
        if not np.isfinite(f):
            continue
        f2, g2, Hp = p.eval_with_hessian_proj(x)
        vs = np.unique(t.handles[e])
        idx = np.concatenate([[2 * v, 2 * v + 1] for v in vs])
        Hd = H.toarray()[np.ix_(idx, idx)]
        lam, V = np.linalg.eigh(0.5 * (Hd + Hd.T))
        ref = (V * np.maximum(lam, 1e-9)) @ V.T
        assert rel_err(Hp.toarray()[np.ix_(idx, idx)], ref) <= 1e-12


def test_gradient_and_hessian_fd(oracle):
    """Central finite differences of f and g on a small disk."""
    w = meshes.disk_param(10, seed=4)
    p = oracle.Problem.from_workload(w)
    rng = np.random.default_rng(0)
    x = w.x0
    f, g, H = p.eval_with_derivatives(x)
    h = 1e-6
    for _ in range(6):
        dvec = rng.normal(size=x.size)
        fd = (p.eval(x + h * dvec) - p.eval(x - h * dvec)) / (2 * h)
        assert abs(fd - g @ dvec) <= 1e-6 * max(1.0, abs(fd))
        gp = p.eval_with_gradient(x + h * dvec)[1]
        gm = p.eval_with_gradient(x - h * dvec)[1]
        assert rel_err((gp - gm) / (2 * h), H @ dvec) <= 1e-6


def test_disk_newton_converges(oracle):
    """Config 0 (64x64-grid disk): 20 Projected-Newton iterations converge."""
    w = meshes.disk_param(64, seed=0)
    assert 5500 < w.info["n_faces"] < 6500
    p = oracle.Problem.from_workload(w)
    x, fh, _ = p.newton(w.x0, 20)
    assert np.all(np.diff(fh) <= 1e-12 * fh[0])
    assert abs(fh[-1] - fh[-2]) <= 1e-12 * fh[-1]
    f, g, H = p.eval_with_hessian_proj(x)
    assert np.max(np.abs(g)) < 1e-6


def test_line_search_failure_keeps_x(oracle):
    """LineSearch.hh:62-64: no decrease -> x0 returned."""
    w = meshes.planar_test_mesh()
    p = oracle.Problem.from_workload(w)
    f, g, H = p.eval_with_hessian_proj(w.x0)
    xo, fo, ok = p.line_search(w.x0, g, f, g)          # ascent direction
    assert not ok and np.array_equal(xo, w.x0)


def test_bad_handle_raises(oracle):
    """Out-of-range handles throw (Element.hh:159-170) and the problem stays usable."""
    p = oracle.Problem(2, 3)
    p.add_elements(meshes.TAD_ENERGY_POSITION_PENALTY, np.array([[5]]), np.array([[0.0, 0.0, 1.0]]))
    with pytest.raises(oracle.OracleError):
        p.eval(np.zeros(6))


def test_newton_direction_needs_hessian(oracle):
    w = meshes.planar_test_mesh()
    p = oracle.Problem.from_workload(w)
    with pytest.raises(oracle.OracleError):
        p.newton_direction(np.zeros(w.n_vars))


def _converge(oracle, w, x, iters=40):
    """Projected Newton, then two full Newton steps on the exact Hessian (PD at
    the minimum): the Armijo search stalls once the energy decrease drops
    below FP64 resolution, the full steps converge quadratically past it."""
    p = oracle.Problem.from_workload(w)
    x, fh, _ = p.newton(x, iters)
    for _ in range(2):
        f, g, H = p.eval_with_derivatives(x)
        x = x + p.newton_direction(g)
    return x, p


def test_adjoint_matches_fd(oracle):
    """Oracle adjoint dL/d(rest) (LDL^T solve + AD<15> block-restricted mixed
    derivatives, ScalarTestHessianBlock.cc) against central differences of
    re-solved minimisers."""
    w = meshes.disk_param_pinned(10, seed=3)
    xs, p = _converge(oracle, w, w.x0)
    rng = np.random.default_rng(7)
    target = xs + rng.normal(scale=0.01, size=xs.size)
    L = lambda x: 0.5 * np.sum((x - target) ** 2)  # noqa: E731
    grad, lam = p.adjoint_rest_gradient(xs, xs - target, w.rest, projected=False)
    h = 1e-5
    for _ in range(3):
        dP = rng.normal(size=w.rest.shape)
        dP /= np.linalg.norm(dP)
        xp, _ = _converge(oracle, meshes.with_rest(w, w.rest + h * dP), xs, 8)
        xm, _ = _converge(oracle, meshes.with_rest(w, w.rest - h * dP), xs, 8)
        fd = (L(xp) - L(xm)) / (2 * h)
        an = float(np.sum(grad * dP))
        assert abs(fd - an) <= 1e-6 * max(abs(fd), 1e-3), (fd, an)
