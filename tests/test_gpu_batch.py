"""Batched Projected Newton (tad_batch_*): meshes of uneven sizes solved in
one problem, one launch per stage, one CUDA graph per iteration.  Each mesh
must reach the energy of its own single-problem solve and of the oracle."""
import numpy as np
import pytest

from tinyad_gb300 import meshes

pytestmark = pytest.mark.gpu


def _meshes():
    return [meshes.disk_param(g, seed=100 + i) for i, g in enumerate((8, 14, 20, 11, 24))]


@pytest.mark.parametrize("chunking", [None, (32, 64)])
@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 1e-5)])
def test_batch_matches_single_solves(tad, oracle, precision, tol, chunking):
    """chunking (32 block rows, 64 threads) splits every mesh over several
    chunks, so the per-mesh reductions combine partials of many blocks"""
    ws = _meshes()
    b = tad.Batch(ws, precision=precision, pcg_rel_tol=tol, pcg_max_iters=400)
    if chunking:
        b.set_chunking(*chunking)
    x, fh = b.newton_solve(b.x0(), 40)
    assert fh.shape == (41, len(ws))
    assert np.all(np.isfinite(fh))
    for m, (w, xm) in enumerate(zip(ws, b.split(x))):
        p = oracle.Problem.from_workload(w)
        xo, fho, _ = p.newton(w.x0, 40)
        f_batch = p.eval(xm)
        assert abs(fh[-1, m] - f_batch) <= 1e-10 * abs(f_batch)
        assert abs(f_batch - fho[-1]) <= 1e-8 * abs(fho[-1]), (m, f_batch, fho[-1])
        assert np.all(np.diff(fh[:, m]) <= 1e-12 * fh[0, m])    # monotone per mesh


def test_batch_deterministic_and_autotune(tad):
    """A fixed launch shape reproduces bit for bit.  Another shape groups the
    per-mesh partial sums differently; CG iterates carry such rounding
    differences into where each inexact solve stops, so trajectories of
    different shapes agree only to the solve tolerance, and what is compared
    across shapes is convergence (test_batch_matches_single_solves with and
    without chunking)."""
    import torch
    ws = _meshes()
    b = tad.Batch(ws, precision=1, pcg_rel_tol=1e-3, pcg_max_iters=64)
    x1, f1 = b.newton_solve(b.x0(), 5)
    x2, f2 = b.newton_solve(b.x0(), 5)
    assert np.array_equal(x1, x2) and np.array_equal(f1, f2)
    xd = torch.from_numpy(b.x0()).cuda()
    best = b.autotune(xd.data_ptr())
    assert best["chunk_rows"] in (256, 512, 1024, 2048, 4096) and best["threads"] in (128, 256)
    assert best["ms_per_iteration"] > 0
    x3, f3 = b.newton_solve(b.x0(), 5)
    x4, f4 = b.newton_solve(b.x0(), 5)
    assert np.array_equal(x3, x4) and np.array_equal(f3, f4)
    b.set_chunking(32, 64)
    x5, f5 = b.newton_solve(b.x0(), 5)
    x6, f6 = b.newton_solve(b.x0(), 5)
    assert np.array_equal(x5, x6) and np.array_equal(f5, f6)
    assert np.all(f5[-1] < f5[0])
    with pytest.raises(tad.TinyADError):
        b.set_chunking(16, 64)


def test_batch_mesh_without_elements(tad, oracle):
    """A mesh with handles but no elements (zero energy and gradient, no
    Hessian blocks) rides along: its variables come back unchanged, its
    energy stays 0, and the other meshes converge as they do alone.  The
    launch shape is set before the first solve."""
    ws = _meshes()[:3]
    t0 = ws[0].terms[0]
    empty = meshes.Workload(name="empty", var_dim=2, n_handles=7, x0=np.linspace(0.0, 1.0, 14),
                            terms=[meshes.Term(t0.energy, t0.valence, np.zeros((0, t0.valence), np.int32),
                                               np.zeros((0, t0.params.shape[1])))])
    ws = [ws[0], empty, ws[1], ws[2]]
    b = tad.Batch(ws, precision=1, pcg_rel_tol=1e-5, pcg_max_iters=400)
    b.set_chunking(32, 64)
    x, fh = b.newton_solve(b.x0(), 40)
    xs = b.split(x)
    assert np.array_equal(xs[1], empty.x0)
    assert np.all(fh[:, 1] == 0.0)
    for m in (0, 2, 3):
        w = ws[m]
        p = oracle.Problem.from_workload(w)
        _, fho, _ = p.newton(w.x0, 40)
        assert abs(p.eval(xs[m]) - fho[-1]) <= 1e-8 * abs(fho[-1]), (m, p.eval(xs[m]), fho[-1])


def test_batch_history_is_each_iterates_energy(tad, oracle):
    """The per-iteration energies the batch reports (the history: f_start
    and the adopted trial energies) are the energies of the batch's own
    iterates, iteration by iteration, including iterations where one mesh
    rejects its full Newton step while the others take theirs: the middle
    mesh starts stretched eight times along v, and its first full steps are
    rejected (checked on the single-problem loop's trial counts).  Each
    mesh's history also follows the single-problem loop with the same
    algorithm (block-Jacobi PCG, 16 Armijo trials).  The two sum their SpMVs
    in different orders, so the solves are tight (1e-10): at 1e-6 the
    different Krylov iterates already move the first step's energy by 2e-5.
    The meshes have two pinned boundary vertices, so the solves are well
    posed (on an unconstrained disk the rotation a tight solve leaves in the
    step depends on the summation order)."""
    base = [meshes.disk_param_pinned(g, seed=100 + i) for i, g in enumerate((8, 14, 20))]
    w1 = base[1]
    x_str = (w1.x0.reshape(-1, 2) * np.array([1.0, 8.0])).ravel()
    ws = [base[0], meshes.Workload(name="stretched", var_dim=2, n_handles=w1.n_handles, x0=x_str, terms=w1.terms),
          base[2]]
    settings = dict(precision=0, pcg_rel_tol=1e-10, pcg_max_iters=2000)
    b = tad.Batch(ws, **settings)
    _, fh = b.newton_solve(b.x0(), 6)
    ps = [oracle.Problem.from_workload(w) for w in ws]
    for k in range(1, 7):
        xk, fk = b.newton_solve(b.x0(), k)      # the same trajectory, stopped after k iterations
        assert np.array_equal(fk, fh[:k + 1])
        for m, xm in enumerate(b.split(xk)):
            e = ps[m].eval(xm)
            assert abs(fh[k, m] - e) <= 1e-12 * abs(e), (k, m, fh[k, m], e)
    rejected = 0
    for m, w in enumerate(ws):
        fn = tad.ScalarFunction.from_workload(w, preconditioner=0, ls_max_iters=16, **settings)
        x = w.x0.copy()
        hist = [fn.eval(x)]
        for _ in range(6):
            x, f1 = fn.newton_solve(x, 1)
            if m == 1 and fn.last_solve_stats()["ls_trials"] > 1:
                rejected += 1
            hist.append(float(f1[-1]))
        assert np.allclose(fh[:, m], hist, rtol=1e-7, atol=0.0), (m, fh[:, m], hist)
    assert rejected >= 1
