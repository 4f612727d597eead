"""ORACLE -- test infrastructure only.  Not part of the product.

ctypes front end of the CPU restatement in oracle/oracle.cpp.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module,
and only as the parity reference / the timed CPU baseline.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(_HERE, "ad_scalar.hh"))):
        subprocess.check_call(["sh", os.path.join(_HERE, "build.sh")])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.oracle_last_error.restype = ctypes.c_char_p
        L.oracle_problem_create.restype = ctypes.c_void_p
        L.oracle_problem_create.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int]
        L.oracle_problem_destroy.argtypes = [ctypes.c_void_p]
        L.oracle_add_elements.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int64, _ip, _dp, ctypes.c_int]
        L.oracle_eval.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.oracle_eval_with_gradient.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.oracle_eval_with_hessian.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_double, _dp, _dp, _i64p]
        L.oracle_get_hessian.argtypes = [ctypes.c_void_p, _ip, _ip, _dp]
        L.oracle_newton_direction.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, _dp]
        L.oracle_line_search.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double, _dp, ctypes.c_double, _dp, _dp]
        L.oracle_newton.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_double, _dp, _dp]
        L.oracle_prepare_solver.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double]
        L.oracle_n_threads.argtypes = [ctypes.c_void_p]
        L.oracle_adjoint_rest_gradient.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_int, ctypes.c_double, _dp, _dp]
        for name in ("oracle_scalar_unary", "oracle_scalar_binary"):
            if hasattr(L, name):
                pass
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def newton_decrement(d, g) -> float:
    """newton_decrement(d, g) = -0.5 d.g (include/TinyAD/Utils/NewtonDecrement.hh:20-26)."""
    return -0.5 * float(np.dot(np.asarray(d, np.float64), np.asarray(g, np.float64)))


class OracleError(RuntimeError):
    pass


class Problem:
    """CPU restatement of ScalarFunction (include/TinyAD/ScalarFunction.hh)."""

    def __init__(self, var_dim: int, n_handles: int, n_threads: int = -1):
        self.L = lib()
        self.var_dim = var_dim
        self.n_vars = var_dim * n_handles
        self.h = self.L.oracle_problem_create(var_dim, n_handles, n_threads)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.oracle_problem_destroy(self.h)
            self.h = None

    def _check(self, rc):
        if rc != 0 and rc != 4:
            raise OracleError(self.L.oracle_last_error().decode())
        return rc

    @property
    def n_threads(self) -> int:
        return self.L.oracle_n_threads(self.h)

    def add_elements(self, energy: int, handles: np.ndarray, params: np.ndarray):
        handles = np.ascontiguousarray(handles, np.int32)
        params = np.ascontiguousarray(params, np.float64)
        n, N = handles.shape
        self._check(self.L.oracle_add_elements(self.h, energy, N, n, handles.ctypes.data_as(_ip), _d(params),
                                               params.shape[1] if params.ndim == 2 else 0))

    @classmethod
    def from_workload(cls, w, n_threads: int = -1) -> "Problem":
        p = cls(w.var_dim, w.n_handles, n_threads)
        for t in w.terms:
            p.add_elements(t.energy, t.handles, t.params)
        return p

    def eval(self, x) -> float:
        x = np.ascontiguousarray(x, np.float64)
        f = np.zeros(1)
        self._check(self.L.oracle_eval(self.h, _d(x), _d(f)))
        return float(f[0])

    def eval_with_gradient(self, x):
        x = np.ascontiguousarray(x, np.float64)
        f = np.zeros(1)
        g = np.zeros(self.n_vars)
        self._check(self.L.oracle_eval_with_gradient(self.h, _d(x), _d(f), _d(g)))
        return float(f[0]), g

    def _hessian(self, x, project, eps):
        import scipy.sparse as sp
        x = np.ascontiguousarray(x, np.float64)
        f = np.zeros(1)
        g = np.zeros(self.n_vars)
        nnz = np.zeros(1, np.int64)
        self._check(self.L.oracle_eval_with_hessian(self.h, _d(x), int(project), eps, _d(f), _d(g),
                                                    nnz.ctypes.data_as(_i64p)))
        outer = np.zeros(self.n_vars + 1, np.int32)
        inner = np.zeros(int(nnz[0]), np.int32)
        vals = np.zeros(int(nnz[0]))
        self.L.oracle_get_hessian(self.h, outer.ctypes.data_as(_ip), inner.ctypes.data_as(_ip), _d(vals))
        H = sp.csc_matrix((vals, inner, outer), shape=(self.n_vars, self.n_vars))
        return float(f[0]), g, H

    def eval_with_derivatives(self, x):
        return self._hessian(x, False, 0.0)

    def eval_with_hessian_proj(self, x, eps: float = 1e-9):
        return self._hessian(x, True, eps)

    def newton_direction(self, g, w: float = 0.0):
        """d = -(H + wI)^-1 g for the Hessian of the last eval_with_hessian_proj /
        eval_with_derivatives call."""
        g = np.ascontiguousarray(g, np.float64)
        d = np.zeros(self.n_vars)
        self._check(self.L.oracle_newton_direction(self.h, _d(g), w, _d(d)))
        return d

    def line_search(self, x, d, f, g, s_max: float = 1.0):
        x = np.ascontiguousarray(x, np.float64)
        d = np.ascontiguousarray(d, np.float64)
        g = np.ascontiguousarray(g, np.float64)
        xo = np.zeros(self.n_vars)
        fo = np.zeros(1)
        rc = self._check(self.L.oracle_line_search(self.h, _d(x), _d(d), f, _d(g), s_max, _d(xo), _d(fo)))
        return xo, float(fo[0]), rc == 0

    def adjoint_rest_gradient(self, x, dLdx, rest, projected: bool = True, eps: float = 1e-9):
        """dL/d(rest positions) by an LDL^T adjoint solve and AD<15> mixed blocks."""
        x, dLdx = np.ascontiguousarray(x, np.float64), np.ascontiguousarray(dLdx, np.float64)
        rest = np.ascontiguousarray(rest, np.float64).reshape(-1)
        out = np.zeros(rest.size)
        lam = np.zeros(self.n_vars)
        self._check(self.L.oracle_adjoint_rest_gradient(self.h, _d(x), _d(dLdx), _d(rest), int(projected), eps,
                                                        _d(out), _d(lam)))
        return out.reshape(-1, 3), lam

    def prepare_solver(self, x, eps: float = 1e-9):
        """The linear solver's pattern analysis (Hessian sparsity, ordering,
        symbolic LDL^T) at x, which the reference caches across Newton
        iterations (LinearSolver.hh:12-19); later newton() calls only factorise."""
        x = np.ascontiguousarray(x, np.float64)
        self._check(self.L.oracle_prepare_solver(self.h, _d(x), eps))

    def newton(self, x, iters: int, eps: float = 1e-9):
        """Projected Newton as in tests/NewtonTest.cc:69-75; returns (x, f_hist, times)."""
        x = np.ascontiguousarray(x, np.float64).copy()
        fh = np.zeros(iters + 1)
        times = np.zeros(4)
        self._check(self.L.oracle_newton(self.h, _d(x), iters, eps, _d(fh), _d(times)))
        return x, fh, times
