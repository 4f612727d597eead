"""torch.autograd.Function around the library's adjoint -- test harness only.

forward(rest): solves x*(rest) = argmin E(x, rest) on the device (Projected
Newton, then full Newton steps on the exact Hessian) and returns the loss
L = 0.5 |x* - target|^2; backward returns dL/d(rest) from
tad_adjoint_rest_gradient.
"""
import numpy as np
import torch

import tinyad_gb300 as tad
from tinyad_gb300 import meshes


def solve_min(w, x0, newton_iters=30, full_steps=2, tol=1e-13):
    return tad.solve_minimiser(w, x0, newton_iters, full_steps, tol)


class RestShapeLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rest, w, x0, target):
        wr = meshes.with_rest(w, rest.detach().cpu().numpy())
        x, fn = solve_min(wr, x0)
        ctx.save_for_backward(rest)
        ctx.state = (wr, x, target, fn)
        return rest.new_tensor(0.5 * float(np.sum((x - target) ** 2)))

    @staticmethod
    def backward(ctx, grad_out):
        (rest,) = ctx.saved_tensors
        wr, x, target, fn = ctx.state
        g, lam, it = fn.adjoint_rest_gradient(x, x - target, wr.rest, projected=False)
        return grad_out * rest.new_tensor(g), None, None, None
