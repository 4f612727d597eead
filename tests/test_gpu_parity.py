"""GPU parity tests: the CUDA path through the C ABI against the oracle (the
CPU restatement of TinyAD's path) on the same seeded inputs.

Tolerances (FP64 path): f, g and H within 1e-10 normwise relative error
(max |a - b| / max |b|); final Newton energy within 1e-8 relative.
"""
import json
import os

import numpy as np
import pytest

from conftest import rel_err, sparse_rel_err, torus_mesh, valid_perturbation
from tinyad_gb300 import meshes

pytestmark = pytest.mark.gpu

TOL = 1e-10
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")


def _pair(tad, oracle, w, **kw):
    return tad.ScalarFunction.from_workload(w, **kw), oracle.Problem.from_workload(w)


def test_known_answers_device(tad):
    """Operator known answers (tests/ScalarTest{Unary,Binary}Operators.cc) on
    the device Double<1>, and on Mixed<1> (FP32 derivatives) at FP32 accuracy."""
    for c in json.load(open(GOLDEN)):
        exp = np.asarray(c["expected"])
        scale = max(1.0, np.max(np.abs(exp)))
        got = tad.debug_scalar_op(c["op"], c["a"], c["b"], tad.PREC_FP64)
        np.testing.assert_allclose(got, exp, rtol=0, atol=c["tol"] * scale, err_msg=f'{c["name"]} ({c["source"]})')
        got = tad.debug_scalar_op(c["op"], c["a"], c["b"], tad.PREC_MIXED)
        np.testing.assert_allclose(got, exp, rtol=0, atol=max(c["tol"], 2e-6) * scale, err_msg=c["name"])


def test_mixed_value_conversions(tad):
    """The mixed scalar's double-float value channel: double -> hi + lo on the
    device is a bit-level split without FP64 instructions.  A round trip
    through `a + 0` (op 29) must return the input within 2^-47 relative in
    the normal float range, give a signed zero below it and inf above it,
    keep signed zero, and propagate inf / NaN."""
    rng = np.random.default_rng(5)
    vals = list(np.ldexp(rng.uniform(-1, 1, 200), rng.integers(-70, 70, 200)))
    vals += [1.0, -1.0, 0.1, 1.0 / 3.0, 2.0 ** -74, 2.0 ** -75, 1e-30, -1e-40, 1e-300, 3.0e38, -3.4e38, 1e39,
             1e300, np.nextafter(1.0, 2.0), 5e-324]
    for v in vals:
        got = tad.debug_scalar_op(29, (v, 1.0, 0.0), (0.0, 0.0, 0.0), tad.PREC_MIXED)[0]
        if abs(v) < 2.0 ** -126:
            # below the normal float range the double-float cannot hold the value
            # (the conversion gives a signed zero; `+ 0` then yields +0)
            assert got == 0.0, (v, got)
        elif abs(v) > 3.4e38:
            with np.errstate(over="ignore"):
                as_float = np.float64(np.float32(v))
            assert got == as_float or abs(got - v) <= 2.0 ** -47 * abs(v), (v, got)
        else:
            assert abs(got - v) <= 2.0 ** -47 * abs(v), (v, got)
    z = tad.debug_scalar_op(0, (0.0, 1.0, 0.0), (0.0, 0.0, 0.0), tad.PREC_MIXED)[0]   # -(+0) = -0
    assert z == 0.0 and np.signbit(z)
    assert tad.debug_scalar_op(29, (np.inf, 1.0, 0.0), (0.0, 0.0, 0.0), tad.PREC_MIXED)[0] == np.inf
    assert np.isnan(tad.debug_scalar_op(29, (np.nan, 1.0, 0.0), (0.0, 0.0, 0.0), tad.PREC_MIXED)[0])


def _quad(A, b, c):
    return np.concatenate([np.asarray(A, float).ravel(), np.asarray(b, float), [c]])[None, :]


def test_scalar_function_quadratics(tad):
    """tests/ScalarFunctionTest.cc:10-151 on the device."""
    f1 = tad.ScalarFunction(1, 1)
    f1.add_elements(meshes.TAD_ENERGY_QUADRATIC, [[0]], _quad([[2.0]], [1.0], 1.0))
    f, g, H = f1.eval_with_hessian_proj(np.array([1.0]))
    assert f == 4.0 and g[0] == 5.0 and H[0, 0] == 4.0
    A2 = [[2.0, 1.0], [1.0, 1.0]]
    f2 = tad.ScalarFunction(2, 1)
    f2.add_elements(meshes.TAD_ENERGY_QUADRATIC, [[0]], _quad(A2, [1.0, 0.0], 1.0))
    x = np.array([1.0, 2.0])
    assert f2.eval(x) == 12.0
    fg, gg = f2.eval_with_gradient(x)
    assert fg == 12.0 and list(gg) == [9.0, 6.0]
    for f, g, H in (f2.eval_with_derivatives(x), f2.eval_with_hessian_proj(x)):
        assert f == 12.0 and list(g) == [9.0, 6.0]
        assert np.array_equal(H.toarray(), [[4.0, 2.0], [2.0, 2.0]])
    f3 = tad.ScalarFunction(2, 1)
    f3.add_elements(meshes.TAD_ENERGY_QUADRATIC, [[0]], _quad(-np.array(A2), [-1.0, 0.0], -1.0))
    f, g, H = f3.eval_with_derivatives(x)
    assert f == -12.0 and list(g) == [-9.0, -6.0] and np.array_equal(H.toarray(), [[-4.0, -2.0], [-2.0, -2.0]])
    f, g, Hp = f3.eval_with_hessian_proj(x)
    assert np.all(np.linalg.eigvalsh(Hp.toarray()) > 0)


def test_planar_newton(tad, oracle):
    """tests/NewtonTest.cc:57-111 on the device: nnz formula, f -> 4 and
    g -> 0, same final energy as the oracle, bitwise deterministic."""
    w = meshes.planar_test_mesh()
    fn, p = _pair(tad, oracle, w, pcg_rel_tol=1e-14, pcg_max_iters=200)
    f, g, H = fn.eval_with_hessian_proj(w.x0)
    assert H.nnz == 4 * 6 + 8 * (6 + 4 - 1)
    fo, go, Ho = p.eval_with_hessian_proj(w.x0)
    assert rel_err(f, fo) <= TOL and rel_err(g, go) <= TOL and sparse_rel_err(H, Ho) <= TOL
    x, fh = fn.newton_solve(w.x0, 10)
    x2, fh2 = fn.newton_solve(w.x0, 10)
    assert np.array_equal(x, x2) and np.array_equal(fh, fh2)
    f, g, H = fn.eval_with_hessian_proj(x)
    assert abs(fn.eval(x) - f) <= 1e-15
    assert abs(f - 4.0) <= 1e-12
    assert np.max(np.abs(g)) <= 1e-10
    xo, fho, _ = p.newton(w.x0, 10)
    assert abs(fh[-1] - fho[-1]) <= 1e-8 * abs(fho[-1])


def _perturbed(w, scale, seed):
    rng = np.random.default_rng(seed)
    return w.x0 + rng.normal(scale=scale, size=w.x0.size)


@pytest.mark.parametrize("grid", [12, 64])
def test_disk_eval_parity(tad, oracle, grid):
    """f, g, H of eval / eval_with_gradient / eval_with_derivatives /
    eval_with_hessian_proj on the disk parametrisation (config 0 at grid 64)."""
    w = meshes.disk_param(grid, seed=0)
    fn, p = _pair(tad, oracle, w)
    for x in (w.x0, valid_perturbation(w, p, 0.002, 1)):
        assert rel_err(fn.eval(x), p.eval(x)) <= TOL
        f, g = fn.eval_with_gradient(x)
        fo, go = p.eval_with_gradient(x)
        assert rel_err(f, fo) <= TOL and rel_err(g, go) <= TOL
        f, g, H = fn.eval_with_derivatives(x)
        fo, go, Ho = p.eval_with_derivatives(x)
        assert rel_err(f, fo) <= TOL and rel_err(g, go) <= TOL and sparse_rel_err(H, Ho) <= TOL
        assert H.nnz == Ho.nnz
        f, g, H = fn.eval_with_hessian_proj(x)
        fo, go, Ho = p.eval_with_hessian_proj(x)
        assert rel_err(f, fo) <= TOL and rel_err(g, go) <= TOL and sparse_rel_err(H, Ho) <= TOL


def test_inverted_elements(tad, oracle):
    """det <= 0 -> +inf energy, zero derivatives and an eps*I projected block
    (NewtonTest.cc:40-41, HessianProjection.hh:66-98), as in the oracle."""
    w = meshes.disk_param(12, seed=0)
    x = _perturbed(w, 0.2, 2)
    fn, p = _pair(tad, oracle, w)
    f, g, H = fn.eval_with_hessian_proj(x)
    fo, go, Ho = p.eval_with_hessian_proj(x)
    assert f == np.inf and fo == np.inf
    assert rel_err(g, go) <= TOL and sparse_rel_err(H, Ho) <= TOL
    assert fn.eval(x) == np.inf


@pytest.mark.parametrize("d", [1, 2])
def test_projection_paths(tad, oracle, d):
    """Both device projection paths in one term, against the oracle's general
    projection: dense quadratic elements (N = 2) whose Hessian is translation
    invariant (A = P S P, P removing the d translations; deflated
    eigenproblem) and general ones (A = S; listed and projected by the
    general kernel).  FP64 within 1e-10, mixed precision at FP32 accuracy."""
    rng = np.random.default_rng(23 + d)
    n_handles, n_elem, k = 300, 2000, 2 * d
    handles = np.stack([rng.integers(0, n_handles, n_elem), rng.integers(0, n_handles, n_elem)], 1)
    handles[handles[:, 0] == handles[:, 1], 1] = (handles[handles[:, 0] == handles[:, 1], 0] + 1) % n_handles
    Pm = np.eye(k) - np.array([[1.0 / 2 if (i % d) == (j % d) else 0.0 for j in range(k)] for i in range(k)])
    params = []
    n_general = 0
    for e in range(n_elem):
        M = rng.normal(size=(k, k))
        S = M @ np.diag(rng.choice([-1.0, 1.0], k) * 10.0 ** rng.uniform(-2, 1, k)) @ M.T
        if e % 4 == 0:
            A = S
            n_general += 1
        else:
            A = Pm @ S @ Pm
        params.append(np.concatenate([0.5 * (A + A.T).ravel(), rng.normal(size=k), [0.0]]))
    params = np.array(params)
    x = rng.normal(size=d * n_handles)
    p = oracle.Problem(d, n_handles)
    p.add_elements(meshes.TAD_ENERGY_QUADRATIC, handles, params)
    fo, go, Ho = p.eval_with_hessian_proj(x)
    assert n_general > 0
    for prec, tol in ((tad.PREC_FP64, TOL), (tad.PREC_MIXED, 2e-5)):
        fn = tad.ScalarFunction(d, n_handles, precision=prec)
        fn.add_elements(meshes.TAD_ENERGY_QUADRATIC, handles, params)
        f, g, H = fn.eval_with_hessian_proj(x)
        assert rel_err(f, fo) <= TOL and rel_err(g, go) <= TOL
        assert sparse_rel_err(H, Ho) <= tol, (prec, sparse_rel_err(H, Ho))
        # flip mode (eps < 0)
        fo2, go2, Ho2 = p.eval_with_hessian_proj(x, eps=-1.0)
        f2, g2, H2 = fn.eval_with_hessian_proj(x, projection_eps=-1.0)
        assert sparse_rel_err(H2, Ho2) <= tol, (prec, sparse_rel_err(H2, Ho2))


def test_disk_newton_parity(tad, oracle):
    """Config 0: 20 Projected-Newton iterations on the device reach the
    oracle's (LDL^T-based) final energy within 1e-8 relative."""
    w = meshes.disk_param(64, seed=0)
    fn, p = _pair(tad, oracle, w, pcg_rel_tol=1e-10, pcg_max_iters=2000)
    x, fh = fn.newton_solve(w.x0, 20)
    xo, fho, _ = p.newton(w.x0, 20)
    assert abs(fh[-1] - fho[-1]) <= 1e-8 * abs(fho[-1]), (fh, fho)
    assert abs(fn.eval(x) - p.eval(x)) <= TOL * abs(fho[-1])


def test_tet_eval_parity(tad, oracle):
    """k = 12 symmetric Dirichlet tets + penalties (config 1 at 4^3 cells)."""
    w = meshes.tet_twist(4, seed=1)
    fn, p = _pair(tad, oracle, w)
    for x in (w.x0, valid_perturbation(w, p, 0.01, 3)):
        f, g, H = fn.eval_with_hessian_proj(x)
        fo, go, Ho = p.eval_with_hessian_proj(x)
        assert rel_err(f, fo) <= TOL and rel_err(g, go) <= TOL and sparse_rel_err(H, Ho) <= TOL
        f, g, H = fn.eval_with_derivatives(x)
        fo, go, Ho = p.eval_with_derivatives(x)
        assert rel_err(f, fo) <= TOL and rel_err(g, go) <= TOL and sparse_rel_err(H, Ho) <= TOL


def test_tet_mixed_lane_kernels(tad, oracle):
    """Mixed precision on tets runs the lane-split evaluation (three
    double-float gradient lanes and twelve FP32 Hessian lanes per element,
    each on an index triple of the affine plane of order 3): f and g match
    the FP64 oracle, the exact and the projected H match it at FP32
    accuracy, and inverted elements give +inf, zero derivatives and the
    eps*I projected block, as the reference does (HessianProjection.hh:66-98)."""
    w = meshes.tet_twist(4, seed=1)
    fm = tad.ScalarFunction.from_workload(w, precision=tad.PREC_MIXED)
    p = oracle.Problem.from_workload(w)
    for x in (w.x0, valid_perturbation(w, p, 0.01, 3)):
        f, g, H = fm.eval_with_derivatives(x)
        fo, go, Ho = p.eval_with_derivatives(x)
        assert rel_err(f, fo) <= 1e-12 and rel_err(g, go) <= 1e-10, (rel_err(f, fo), rel_err(g, go))
        assert H.nnz == Ho.nnz and sparse_rel_err(H, Ho) <= 5e-5, sparse_rel_err(H, Ho)
        f, g, H = fm.eval_with_hessian_proj(x)
        fo, go, Ho = p.eval_with_hessian_proj(x)
        assert rel_err(f, fo) <= 1e-12 and rel_err(g, go) <= 1e-10
        assert sparse_rel_err(H, Ho) <= 5e-5, sparse_rel_err(H, Ho)
    x = w.x0.copy()
    x[2::3] *= -1.0   # mirrored: every tetrahedron inverted
    assert p.eval(x) == np.inf
    f, g, H = fm.eval_with_hessian_proj(x)
    fo, go, Ho = p.eval_with_hessian_proj(x)
    assert f == np.inf and fo == np.inf
    assert rel_err(g, go) <= 1e-10 and sparse_rel_err(H, Ho) <= 5e-5, (rel_err(g, go), sparse_rel_err(H, Ho))


def test_tet_newton_parity(tad, oracle):
    w = meshes.tet_twist(4, seed=1)
    fn, p = _pair(tad, oracle, w, pcg_rel_tol=1e-10, pcg_max_iters=3000)
    x, fh = fn.newton_solve(w.x0, 40)
    xo, fho, _ = p.newton(w.x0, 40)
    assert abs(fh[-1] - fho[-1]) <= 1e-8 * abs(fho[-1]), (fh[-3:], fho[-3:])


def test_laplacian_device(tad):
    """Hessian of the Dirichlet energy = graph Laplacian (DynamicElementsTest.cc:60-91)."""
    import scipy.sparse as sp
    nv, F = torus_mesh()
    fn = tad.ScalarFunction(1, nv)
    fn.add_elements(meshes.TAD_ENERGY_DIRICHLET_TRI, F, np.full((F.shape[0], 1), 0.25))
    H = fn.eval_hessian_of_quadratic()
    rows, cols, vals = [], [], []
    for t in F:
        for i in range(3):
            rows += [t[i], t[i]]
            cols += [t[i], t[(i + 1) % 3]]
            vals += [1.0, -1.0]
    Lref = sp.coo_matrix((vals, (rows, cols)), shape=(nv, nv)).tocsr()
    Lref.sum_duplicates()
    assert H.nnz == Lref.nnz and abs(H - Lref).max() <= 1e-12


def test_determinism(tad):
    """Bitwise reproducible evaluations and solves (NewtonTest.cc:97-111)."""
    w = meshes.disk_param(40, seed=5)
    fn = tad.ScalarFunction.from_workload(w)
    a = fn.eval_with_hessian_proj(w.x0)
    b = fn.eval_with_hessian_proj(w.x0)
    assert a[0] == b[0] and np.array_equal(a[1], b[1]) and np.array_equal(a[2].data, b[2].data)
    x1, f1 = fn.newton_solve(w.x0, 3)
    x2, f2 = fn.newton_solve(w.x0, 3)
    assert np.array_equal(x1, x2) and np.array_equal(f1, f2)


def test_errors_leave_function_usable(tad):
    """Bad input raises RuntimeError and the function stays usable
    (tests/ExceptionTest.cc:8-53)."""
    fn = tad.ScalarFunction(2, 3)
    with pytest.raises(RuntimeError):
        fn.add_elements(meshes.TAD_ENERGY_POSITION_PENALTY, [[7]], [[0.0, 0.0, 1.0]])
    with pytest.raises(RuntimeError):
        fn.add_elements(meshes.TAD_ENERGY_SYMMETRIC_DIRICHLET_TET, [[0, 1, 2, 0]], np.zeros((1, 10)))
    fn.add_elements(meshes.TAD_ENERGY_POSITION_PENALTY, [[1]], [[1.0, 2.0, 1.0]])
    with pytest.raises(RuntimeError):
        fn.eval(np.zeros(5))
    f, g = fn.eval_with_gradient(np.zeros(6))
    assert f == 5.0 and list(g) == [0.0, 0.0, -2.0, -4.0, 0.0, 0.0]
    with pytest.raises(RuntimeError):
        fn.add_elements(meshes.TAD_ENERGY_POSITION_PENALTY, [[0]], [[1.0, 2.0, 1.0]])   # after finalize


def test_line_search_api(tad, oracle):
    """line_search matches the reference's sequential Armijo search."""
    w = meshes.disk_param(20, seed=6)
    fn, p = _pair(tad, oracle, w)
    f, g, H = fn.eval_with_hessian_proj(w.x0)
    p.eval_with_hessian_proj(w.x0)
    d = p.newton_direction(g)
    x_gpu = fn.line_search(w.x0, d, f, g)
    x_cpu, _, ok = p.line_search(w.x0, d, f, g)
    assert ok and rel_err(x_gpu, x_cpu) <= 1e-14
    x_bad = fn.line_search(w.x0, g, f, g)          # ascent direction: x unchanged
    assert np.array_equal(x_bad, w.x0)


def test_newton_direction_api(tad, oracle):
    """newton_direction (PCG) against the oracle's LDL^T direction."""
    w = meshes.disk_param(20, seed=6)
    fn, p = _pair(tad, oracle, w, pcg_rel_tol=1e-13, pcg_max_iters=5000)
    d, f, g = fn.newton_direction(w.x0)
    fo, go, Ho = p.eval_with_hessian_proj(w.x0)
    do = p.newton_direction(go)
    # the direction solves the oracle's system (it differs from LDL^T's only
    # along the eps-scaled translation null space)
    assert rel_err(Ho @ d, -go) <= 1e-9
    assert rel_err(Ho @ do, -go) <= 1e-9
    assert abs(d @ go - do @ go) <= 1e-8 * abs(do @ go)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_newton_direction_tet_w_identity(tad, oracle, precision):
    """newton_direction with w I added (NewtonDirection.hh:32) on tets, whose
    PCG runs on the sliced-ELL copy of H: in FP64 the direction solves the
    oracle's (H + w I) d = -g; in mixed precision the system of its own FP32
    Hessian (FP64 refinement to 1e-11), whose shifted diagonal H_ii + w is
    itself rounded to FP32 (hence 1e-6 there)."""
    import scipy.sparse as sp
    w = meshes.tet_twist(4, seed=2)
    prec = tad.PREC_MIXED if precision == "mixed" else tad.PREC_FP64
    fn, p = _pair(tad, oracle, w, precision=prec, pcg_rel_tol=1e-11, pcg_max_iters=5000, refine_max_iters=8,
                  refine_rel_tol=1e-11)
    x = valid_perturbation(w, p, 0.01, 4)
    if precision == "fp64":
        _, g_ref, H_ref = p.eval_with_hessian_proj(x)
    else:
        _, g_ref, H_ref = fn.eval_with_hessian_proj(x)
    for wid in (0.0, 0.5):
        d, f, g = fn.newton_direction(x, w_identity=wid)
        A = H_ref + wid * sp.identity(H_ref.shape[0], format="csr")
        tol = 1e-6 if (precision == "mixed" and wid != 0.0) else 1e-8
        assert rel_err(A @ d, -g_ref) <= tol, (wid, rel_err(A @ d, -g_ref))


def test_newton_decrement(tad, oracle):
    """newton_decrement (NewtonDecrement.hh:20-26) through the C ABI, host and
    device forms, against the oracle's -d.g/2; and the reference's loop
    (eval_with_hessian_proj -> newton_direction -> stop if the decrement is
    below eps -> line_search) run with the library's calls and with the
    oracle's stops after the same number of steps, as tad_newton_solve with
    stop_decrement does (the test is taken before the step)."""
    import torch
    w = meshes.disk_param_pinned(12, seed=3)
    fn, p = _pair(tad, oracle, w, pcg_rel_tol=1e-13, pcg_max_iters=5000)
    d, f, g = fn.newton_direction(w.x0)
    dec = fn.newton_decrement(d, g)
    assert dec > 0.0 and abs(dec - oracle.newton_decrement(d, g)) <= 1e-14 * abs(dec)
    dd, gd = torch.from_numpy(d).cuda(), torch.from_numpy(g).cuda()
    assert fn.newton_decrement_device(dd.data_ptr(), gd.data_ptr()) == dec   # same fixed-order reduction
    assert fn.newton_decrement(d, g) == dec                                   # bitwise reproducible
    thr = 1e-12

    def loop(eval_h, direction, decrement, search):
        x, decs = w.x0.copy(), []
        for _ in range(40):
            f, g = eval_h(x)
            d = direction(x, g)
            decs.append(decrement(d, g))
            if decs[-1] < thr:
                break
            x = search(x, d, f, g)
        return x, decs

    def gpu_eval(x):
        f, g, _ = fn.eval_with_hessian_proj(x)
        return f, g

    def cpu_eval(x):
        f, g, _ = p.eval_with_hessian_proj(x)
        return f, g

    xg, dg = loop(gpu_eval, lambda x, g: fn.newton_direction(x)[0], fn.newton_decrement,
                  lambda x, d, f, g: fn.line_search(x, d, f, g))
    xc, dc = loop(cpu_eval, lambda x, g: p.newton_direction(g), oracle.newton_decrement,
                  lambda x, d, f, g: p.line_search(x, d, f, g)[0])
    assert 2 < len(dc) < 40 and len(dg) == len(dc)
    for a, b in zip(dg, dc):
        if b > 1e-6:
            assert abs(a - b) <= 1e-7 * b
    assert rel_err(xg, xc) <= 1e-8
    # the fused loop: the same number of steps, the same minimiser
    steps = len(dc) - 1
    x, fh = fn.newton_solve(w.x0, 40, stop_decrement=thr)
    assert len(fh) - 1 == steps
    assert rel_err(x, xc) <= 1e-8 and abs(fh[-1] - p.eval(xc)) <= 1e-12 * abs(fh[-1])


def test_mixed_precision(tad, oracle):
    """Mixed mode: FP32 element Hessians, projection and PCG; double-float
    (~48-bit) values (edge vectors, determinant, inverse, energy) and
    gradient in the element kernel; FP64 line-search energy and refinement
    residuals.  f and g match the FP64 oracle, H carries FP32 rounding, and
    the Newton loop reaches the FP64 final energy within 1e-8 relative."""
    w = meshes.disk_param(64, seed=0)
    fm = tad.ScalarFunction.from_workload(w, precision=tad.PREC_MIXED, pcg_rel_tol=1e-8, pcg_max_iters=2000)
    p = oracle.Problem.from_workload(w)
    x = w.x0
    f, g, H = fm.eval_with_hessian_proj(x)
    fo, go, Ho = p.eval_with_hessian_proj(x)
    assert rel_err(f, fo) <= 1e-12
    assert rel_err(g, go) <= 1e-10
    assert sparse_rel_err(H, Ho) <= 5e-5
    xm, fhm = fm.newton_solve(w.x0, 25)
    xo, fho, _ = p.newton(w.x0, 25)
    assert abs(fhm[-1] - fho[-1]) <= 1e-8 * abs(fho[-1]), (fhm[-4:], fho[-4:])


def test_newton_direction_reduced_basis_switch_solver(tad):
    """tests/SwitchSolverTest.cc:16-36: x^2 + y^2 at (1, 1) with B = I gives
    the Newton step (-1, -1)."""
    import scipy.sparse as sp
    f1 = tad.ScalarFunction(2, 1)
    f1.add_elements(meshes.TAD_ENERGY_QUADRATIC, [[0]], _quad([[1.0, 0.0], [0.0, 1.0]], [0.0, 0.0], 0.0))
    d, f, g = f1.newton_direction_reduced_basis(np.array([1.0, 1.0]), sp.identity(2, format="csr"))
    assert f == 2.0 and np.all(g == 2.0)
    assert np.all(np.abs(d + 1.0) <= 1e-15)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("mixed", 1e-4)])
@pytest.mark.parametrize("w_identity", [0.0, 0.5])
def test_newton_direction_reduced_basis_pinned_boundary(tad, oracle, precision, tol, w_identity):
    """newton_direction_reduced_basis (NewtonDirection.hh:76-123) with B the
    free (interior) coordinates of a disk parametrisation whose boundary is
    fixed: d = B (B^T H B + w I)^-1 (-B^T g) against a direct solve of the
    reduced system assembled from the oracle's projected Hessian."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    w = meshes.disk_param(24, seed=3)
    prec = tad.PREC_MIXED if precision == "mixed" else tad.PREC_FP64
    fn = tad.ScalarFunction.from_workload(w, precision=prec, pcg_rel_tol=1e-12, pcg_max_iters=5000)
    p = oracle.Problem.from_workload(w)
    x = w.x0
    F = np.asarray(w.terms[0].handles)
    edges = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
    uniq, counts = np.unique(edges, axis=0, return_counts=True)
    boundary = np.unique(uniq[counts == 1])
    free_v = np.setdiff1d(np.arange(w.n_handles), boundary)
    free = np.sort(np.concatenate([2 * free_v, 2 * free_v + 1]))
    B = sp.csr_matrix((np.ones(free.size), (free, np.arange(free.size))), shape=(w.n_vars, free.size))
    d, f, g = fn.newton_direction_reduced_basis(x, B, w_identity=w_identity)
    fo, go, Ho = p.eval_with_hessian_proj(x)
    Hr = (B.T @ Ho @ B + w_identity * sp.identity(free.size)).tocsc()
    d_ref = B @ spla.spsolve(Hr, -(B.T @ go))
    assert rel_err(f, fo) <= 1e-12
    assert rel_err(d, d_ref) <= tol
    assert np.all(d[2 * boundary] == 0.0) and np.all(d[2 * boundary + 1] == 0.0)


@pytest.mark.parametrize("precision", ["fp64"])
def test_amg_preconditioned_solve(tad, precision):
    """A solve that block-Jacobi PCG cannot finish in its first iterations
    restarts with the AMG-preconditioned CG (preconditioner = 1): near the
    minimiser of a pinned disk parametrisation (the adjoint's regime) the
    direction solves H d = -g to the tolerance and equals the block-Jacobi
    one, in far fewer iterations."""
    w = meshes.disk_param_pinned(96, seed=4)
    xs, _ = tad.solve_minimiser(w, w.x0)
    x = xs + np.random.default_rng(3).normal(scale=1e-3, size=xs.size)
    prec = tad.PREC_MIXED if precision == "mixed" else tad.PREC_FP64
    kw = dict(precision=prec, pcg_rel_tol=1e-10, pcg_max_iters=20000, refine_max_iters=8, refine_rel_tol=1e-10)
    f_j = tad.ScalarFunction.from_workload(w, preconditioner=0, **kw)
    f_a = tad.ScalarFunction.from_workload(w, preconditioner=1, **kw)
    d_j, _, g = f_j.newton_direction(x)
    it_j = f_j.last_solve_stats()["pcg_iters"]
    d_a, _, _ = f_a.newton_direction(x)
    it_a = f_a.last_solve_stats()["pcg_iters"]
    _, _, H = f_j.eval_with_hessian_proj(x)
    assert rel_err(H @ d_a, -g) <= 1e-8
    assert rel_err(d_a, d_j) <= 1e-6
    assert it_a * 3 < it_j, (it_a, it_j)


def test_mixed_newton_step(tad):
    """The mixed path's Newton step against FP64's at the same state, both
    linear solves to 1e-10: the difference is the precision of the FP32
    Hessian (and projection), a few 1e-6 relative here."""
    w = meshes.disk_param_pinned(32, seed=6)
    xs, _ = tad.solve_minimiser(w, w.x0)
    x = xs + np.random.default_rng(8).normal(scale=1e-3, size=xs.size)
    kw = dict(pcg_rel_tol=1e-10, pcg_max_iters=20000, refine_max_iters=8, refine_rel_tol=1e-10)
    f64 = tad.ScalarFunction.from_workload(w, precision=tad.PREC_FP64, **kw)
    fmx = tad.ScalarFunction.from_workload(w, precision=tad.PREC_MIXED, **kw)
    d64, _, g = f64.newton_direction(x)
    dmx, _, _ = fmx.newton_direction(x)
    _, _, H = f64.eval_with_hessian_proj(x)
    assert rel_err(H @ d64, -g) <= 1e-9
    assert rel_err(dmx, d64) <= 1e-4


def test_mixed_tight_newton_unconstrained(tad):
    """Mixed precision with tight inner solves on an unconstrained disk.  The
    eps-regularised rigid motions make H nearly singular, and the FP32-evaluated
    Hessian is indefinite at its rounding level along them, so a 1e-8 linear
    solve can stop short there (the iterative refinement then returns its best
    iterate; the rigid part of such a step is arbitrary in any precision).  The
    Newton iteration must still reach the FP64 path's minimum energy."""
    w = meshes.disk_param(48, seed=13)
    kw = dict(pcg_rel_tol=1e-8, pcg_max_iters=20000, refine_max_iters=8, refine_rel_tol=1e-8)
    f64 = tad.ScalarFunction.from_workload(w, precision=tad.PREC_FP64, **kw)
    fmx = tad.ScalarFunction.from_workload(w, precision=tad.PREC_MIXED, **kw)
    _, fh64 = f64.newton_solve(w.x0, 30)
    xm, fhmx = fmx.newton_solve(w.x0, 30)
    assert abs(fhmx[-1] - fh64[-1]) <= 1e-8 * abs(fh64[-1]), (fhmx[-1], fh64[-1])
    # the function stays usable after such solves
    f, g, _ = fmx.eval_with_hessian_proj(xm)
    assert np.isfinite(f) and np.all(np.isfinite(g))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_newton_calls_continue(tad, precision):
    """A solve stepped one call per iteration (the library then carries the
    derivatives its speculative full step assembled into the next call) ends
    where one multi-iteration call ends; an evaluation between calls, or a
    changed x, falls back to evaluating at the call's start."""
    w = meshes.disk_param(48, seed=3)
    prec = tad.PREC_MIXED if precision == "mixed" else tad.PREC_FP64
    kw = dict(precision=prec, pcg_rel_tol=1e-2, pcg_max_iters=2000, forcing=0)
    fa = tad.ScalarFunction.from_workload(w, **kw)
    fb = tad.ScalarFunction.from_workload(w, **kw)
    xa, fha = fa.newton_solve(w.x0, 12)
    xb = w.x0.copy()
    fhb = []
    for it in range(12):
        if it == 6:
            fb.eval_with_hessian_proj(xb)      # other evaluations invalidate the carried derivatives
        if it == 9:
            xb = xb + 0.0                      # same values: still a continuation
        xb, fh = fb.newton_solve(xb, 1)
        fhb.append(fh[0])
    fhb.append(fh[-1])
    assert rel_err(xb, xa) <= 1e-12, rel_err(xb, xa)
    assert rel_err(np.array(fhb), fha) <= 1e-12
    # a changed x is not a continuation: the call evaluates at its own start
    xc = xb.copy()
    xc[0] += 1e-7
    xc2, fhc = fb.newton_solve(xc, 1)
    assert abs(fhc[0] - fb.eval(xc)) <= 1e-12 * abs(fhc[0])
    # zero iterations return x as given, whether or not the call would have continued
    xs, _ = fb.newton_solve(xc2, 1)
    xz = xs.copy()
    xz[1] += 1e-7
    xr, _ = fb.newton_solve(xz, 0)
    assert np.array_equal(xr, xz)
    xr2, _ = fb.newton_solve(xr, 0)
    assert np.array_equal(xr2, xz)
    # and the next iteration starts from an evaluation at that x, not from
    # derivatives carried from before it
    _, fhz = fb.newton_solve(xr2, 1)
    assert abs(fhz[0] - fb.eval(xz)) <= 1e-12 * abs(fhz[0])
