"""GPU tests of the rest-shape adjoint (tad_adjoint_rest_gradient): against
the oracle's LDL^T/AD<15> adjoint, and against central finite differences of
re-solved minimisers through the torch.autograd.Function harness."""
import numpy as np
import pytest
import torch

from conftest import rel_err
from tinyad_gb300 import meshes

pytestmark = pytest.mark.gpu


def test_adjoint_vs_oracle(tad, oracle):
    from adjoint_fn import solve_min
    w = meshes.disk_param_pinned(24, seed=3)
    x, fn = solve_min(w, w.x0)
    rng = np.random.default_rng(1)
    target = x + rng.normal(scale=0.01, size=x.size)
    p = oracle.Problem.from_workload(w)
    for projected in (False, True):
        g_gpu, lam_gpu, it = fn.adjoint_rest_gradient(x, x - target, w.rest, projected=projected)
        g_cpu, lam_cpu = p.adjoint_rest_gradient(x, x - target, w.rest, projected=projected)
        assert rel_err(lam_gpu, lam_cpu) <= 1e-8
        assert rel_err(g_gpu, g_cpu) <= 1e-8


def test_adjoint_vs_fd_autograd(tad):
    """torch.autograd gradient (adjoint backward) against central FD,
    h = 1e-6 relative to the rest-shape scale, random unit directions."""
    from adjoint_fn import RestShapeLoss, solve_min
    w = meshes.disk_param_pinned(16, seed=5)
    x0, _ = solve_min(w, w.x0)
    rng = np.random.default_rng(2)
    target = x0 + rng.normal(scale=0.01, size=x0.size)
    rest = torch.tensor(w.rest, dtype=torch.float64, requires_grad=True)
    L = RestShapeLoss.apply(rest, w, x0, target)
    L.backward()
    grad = rest.grad.numpy()
    h = 1e-6
    for _ in range(4):
        dP = rng.normal(size=w.rest.shape)
        dP /= np.linalg.norm(dP)
        with torch.no_grad():
            Lp = RestShapeLoss.apply(torch.tensor(w.rest + h * dP), w, x0, target).item()
            Lm = RestShapeLoss.apply(torch.tensor(w.rest - h * dP), w, x0, target).item()
        fd = (Lp - Lm) / (2 * h)
        an = float(np.sum(grad * dP))
        assert abs(fd - an) <= 1e-4 * max(abs(fd), 1e-3), (fd, an)
