import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def tad():
    """The CUDA library; GPU tests only."""
    import tinyad_gb300
    tinyad_gb300.load()
    return tinyad_gb300


def rel_err(a, b) -> float:
    """max |a - b| / max |b| (normwise relative error, max-abs norm)."""
    a = np.atleast_1d(np.asarray(a, dtype=np.float64))
    b = np.atleast_1d(np.asarray(b, dtype=np.float64))
    if a.shape != b.shape:
        return float("inf")
    same = (a == b)                       # includes equal infinities
    if np.all(same):
        return 0.0
    fin = np.isfinite(b)
    if not np.all(np.isfinite(a[~same])) or not np.all(fin[~same]):
        return float("inf")
    den = max(float(np.max(np.abs(b[fin]))) if fin.any() else 0.0, 1e-300)
    return float(np.max(np.abs(a - b)[~same])) / den


def sparse_rel_err(A, B) -> float:
    """Normwise relative error of two sparse matrices (max-abs over the union)."""
    D = (A - B).tocoo()
    den = max(float(np.max(np.abs(B.data))) if B.nnz else 0.0, 1e-300)
    return float(np.max(np.abs(D.data))) / den if D.nnz else 0.0


def valid_perturbation(w, oracle_problem, scale: float, seed: int):
    """x0 plus seeded noise, halved until no element inverts."""
    rng = np.random.default_rng(seed)
    noise = rng.normal(size=w.x0.size)
    for _ in range(30):
        x = w.x0 + scale * noise
        if np.isfinite(oracle_problem.eval(x)):
            return x
        scale *= 0.5
    return w.x0


def torus_mesh(n: int = 8, m: int = 6):
    """Closed triangle mesh (torus grid), for the Laplacian pin."""
    F = []
    vid = lambda i, j: (i % n) * m + (j % m)  # noqa: E731
    for i in range(n):
        for j in range(m):
            F.append([vid(i, j), vid(i + 1, j), vid(i + 1, j + 1)])
            F.append([vid(i, j), vid(i + 1, j + 1), vid(i, j + 1)])
    return n * m, np.array(F, np.int32)
