"""tinyad_gb300 -- GB300-native sparse per-element derivative path.

Python mirror of TinyAD's ScalarFunction interface for this path
(include/TinyAD/ScalarFunction.hh:57-248), calling the CUDA library
(libtad.so, C ABI in include/tad.h) through ctypes.  Method names, argument
meanings and error behaviour follow the reference: every failure raises
RuntimeError (the reference throws std::runtime_error, Out.hh:73-79) and the
function stays usable afterwards.

There is no CPU fallback: loading fails loudly when the CUDA library or a
GPU is missing.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import meshes  # noqa: F401  (workload generators)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libtad.so")

TAD_OK = 0
TAD_ERR_ARG = 1
TAD_ERR_NONFINITE = 2
TAD_ERR_PCG_NOCONV = 3
TAD_ERR_LS_FAIL = 4
TAD_ERR_TIMEOUT = 5
TAD_ERR_CUDA = 6
TAD_ERR_STATE = 7
TAD_ERR_TOO_MANY_VARS = 8

PREC_FP64 = 0
PREC_MIXED = 1

default_hessian_projection_eps = 1e-9   # HessianProjection.hh:16

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)


class Settings(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("pcg_max_iters", ctypes.c_int), ("pcg_rel_tol", ctypes.c_double),
                ("refine_max_iters", ctypes.c_int), ("refine_rel_tol", ctypes.c_double),
                ("ls_max_iters", ctypes.c_int), ("ls_shrink", ctypes.c_double), ("ls_armijo", ctypes.c_double),
                ("forcing", ctypes.c_int), ("verbose", ctypes.c_int), ("preconditioner", ctypes.c_int)]


class TinyADError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


_lib = None

# every symbol include/tad.h declares (checked by the CPU tests)
EXPORTS = [
    "tad_newton_direction_reduced_basis", "tad_add_vector_elements", "tad_add_vector_elements_custom", "tad_n_outputs",
    "tad_vec_eval", "tad_vec_jacobian_nnz", "tad_vec_jacobian_pattern", "tad_vec_eval_with_jacobian",
    "tad_vec_hessians_nnz", "tad_vec_eval_with_derivatives", "tad_eval_sum_of_squares_with_derivatives",
    "tad_gauss_newton_direction",
    "tad_settings_default", "tad_last_error_message", "tad_version", "tad_problem_create", "tad_problem_destroy",
    "tad_problem_set_settings", "tad_n_vars", "tad_add_elements", "tad_add_elements_custom", "tad_finalize",
    "tad_hessian_nnz", "tad_hessian_pattern", "tad_eval", "tad_eval_with_gradient", "tad_eval_with_derivatives",
    "tad_eval_with_hessian_proj", "tad_eval_d", "tad_eval_with_hessian_proj_d", "tad_newton_direction",
    "tad_line_search", "tad_newton_decrement", "tad_newton_decrement_d", "tad_newton_solve", "tad_newton_solve_d", "tad_last_solve_stats", "tad_debug_scalar_op",
    "tad_get_stream", "tad_measure_fma_peak", "tad_profile_kernels",
    "tad_launch_count", "tad_adjoint_rest_gradient", "tad_eval_symmetric_dirichlet_tri_noalloc",
    "tad_batch_create", "tad_batch_add_elements", "tad_batch_newton_solve", "tad_batch_newton_solve_d",
    "tad_batch_autotune", "tad_batch_set_chunking", "tad_batch_problem", "tad_batch_destroy",
]


def load(build_if_missing: bool = True):
    """Load libtad.so (building it in-tree with nvcc if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise OSError(f"CUDA library not built: {LIB_PATH}")
        from . import build as _b
        _b.build()
    L = ctypes.CDLL(LIB_PATH)
    L.tad_last_error_message.restype = ctypes.c_char_p
    L.tad_version.restype = ctypes.c_char_p
    L.tad_settings_default.argtypes = [ctypes.POINTER(Settings)]
    L.tad_problem_create.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.POINTER(Settings), ctypes.POINTER(ctypes.c_void_p)]
    L.tad_problem_destroy.argtypes = [ctypes.c_void_p]
    L.tad_problem_set_settings.argtypes = [ctypes.c_void_p, ctypes.POINTER(Settings)]
    L.tad_n_vars.argtypes = [ctypes.c_void_p]
    L.tad_n_vars.restype = ctypes.c_int64
    L.tad_add_elements.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int64, _ip, _dp, ctypes.c_int]
    L.tad_finalize.argtypes = [ctypes.c_void_p]
    L.tad_hessian_nnz.argtypes = [ctypes.c_void_p, _i64p]
    L.tad_hessian_pattern.argtypes = [ctypes.c_void_p, _ip, _ip]
    L.tad_eval.argtypes = [ctypes.c_void_p, _dp, _dp]
    L.tad_eval_with_gradient.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
    L.tad_eval_with_derivatives.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp]
    L.tad_eval_with_hessian_proj.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, _dp, _dp, _dp]
    L.tad_eval_d.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _dp]
    L.tad_eval_with_hessian_proj_d.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, _dp,
                                               ctypes.c_void_p, ctypes.c_void_p]
    L.tad_newton_direction.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_double, _dp, _dp, _dp]
    L.tad_add_vector_elements.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int64, _ip,
                                          _dp, ctypes.c_int]
    L.tad_n_outputs.argtypes = [ctypes.c_void_p]
    L.tad_n_outputs.restype = ctypes.c_int64
    L.tad_vec_eval.argtypes = [ctypes.c_void_p, _dp, _dp]
    L.tad_vec_jacobian_nnz.argtypes = [ctypes.c_void_p, _i64p]
    L.tad_vec_jacobian_pattern.argtypes = [ctypes.c_void_p, _ip, _ip]
    L.tad_vec_eval_with_jacobian.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
    L.tad_vec_hessians_nnz.argtypes = [ctypes.c_void_p, _i64p]
    L.tad_vec_eval_with_derivatives.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _i64p, _ip, _ip, _dp]
    L.tad_eval_sum_of_squares_with_derivatives.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp]
    L.tad_gauss_newton_direction.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, _dp, _dp, _dp]
    L.tad_newton_direction_reduced_basis.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int64, _ip, _ip, _dp, ctypes.c_double,
                                                     ctypes.c_double, _dp, _dp, _dp]
    L.tad_newton_decrement.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
    L.tad_newton_decrement_d.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _dp]
    L.tad_line_search.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double, _dp, ctypes.c_double, _dp, _dp]
    L.tad_newton_solve.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_double, _dp,
                                   ctypes.POINTER(ctypes.c_int)]
    L.tad_newton_solve_d.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                     _dp, ctypes.POINTER(ctypes.c_int)]
    L.tad_last_solve_stats.argtypes = [ctypes.c_void_p, _dp, _i64p, _i64p]
    L.tad_debug_scalar_op.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
    L.tad_get_stream.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
    L.tad_measure_fma_peak.argtypes = [ctypes.c_int, _dp]
    L.tad_profile_kernels.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, _dp]
    L.tad_launch_count.argtypes = [ctypes.c_void_p, _i64p]
    L.tad_batch_create.argtypes = [ctypes.c_int, ctypes.c_int, _i64p, ctypes.POINTER(Settings), ctypes.POINTER(ctypes.c_void_p)]
    L.tad_batch_add_elements.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _i64p, _ip, _dp, ctypes.c_int]
    L.tad_batch_newton_solve.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_double, _dp]
    L.tad_batch_newton_solve_d.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double, _dp]
    L.tad_batch_autotune.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, _dp]
    L.tad_batch_set_chunking.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    L.tad_batch_problem.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
    L.tad_batch_destroy.argtypes = [ctypes.c_void_p]
    L.tad_eval_symmetric_dirichlet_tri_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                           ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
    L.tad_adjoint_rest_gradient.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_int, ctypes.c_double, _dp, _dp,
                                            ctypes.POINTER(ctypes.c_int)]
    _lib = L
    return L


def default_settings(**kw) -> Settings:
    s = Settings()
    load().tad_settings_default(ctypes.byref(s))
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def _d(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class ScalarFunction:
    """A sum of per-element energies over d-dimensional variable handles.

    Mirrors TinyAD::ScalarFunction<d, double, Eigen::Index> for the built-in
    energies (tad_energy in include/tad.h); user functors use the C++ front
    end include/tad/ScalarFunction.cuh.
    """

    def __init__(self, var_dim: int, n_handles: int, settings: Settings | None = None, **kw):
        self.L = load()
        self.var_dim = var_dim
        self.n_handles = n_handles
        self.n_vars = var_dim * n_handles
        self.settings = settings if settings is not None else default_settings(**kw)
        h = ctypes.c_void_p()
        self._check(self.L.tad_problem_create(var_dim, n_handles, ctypes.byref(self.settings), ctypes.byref(h)))
        self.h = h
        self._pattern = None

    def close(self):
        if getattr(self, "h", None):
            self.L.tad_problem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, allow=()) -> int:
        if rc != TAD_OK and rc not in allow:
            raise TinyADError(rc, self.L.tad_last_error_message().decode())
        return rc

    def set_settings(self, **kw):
        for k, v in kw.items():
            setattr(self.settings, k, v)
        self._check(self.L.tad_problem_set_settings(self.h, ctypes.byref(self.settings)))

    # ---- setup -------------------------------------------------------------
    def add_elements(self, energy: int, handles, params):
        """add_elements<N>(range, lambda) for a built-in energy."""
        handles = np.ascontiguousarray(handles, dtype=np.int32)
        if handles.ndim == 1:
            handles = handles[:, None]
        params = _f64(params)
        if params.ndim == 1:
            params = params[:, None]
        n, N = handles.shape
        self._check(self.L.tad_add_elements(self.h, int(energy), N, n, handles.ctypes.data_as(_ip), _d(params),
                                            params.shape[1] if n > 0 else int(params.shape[-1])))
        self._pattern = None

    @classmethod
    def from_workload(cls, w, **kw) -> "ScalarFunction":
        f = cls(w.var_dim, w.n_handles, **kw)
        for t in w.terms:
            f.add_elements(t.energy, t.handles, t.params)
        return f

    def finalize(self):
        self._check(self.L.tad_finalize(self.h))

    def hessian_pattern(self):
        if self._pattern is None:
            nnz = np.zeros(1, np.int64)
            self._check(self.L.tad_hessian_nnz(self.h, nnz.ctypes.data_as(_i64p)))
            outer = np.zeros(self.n_vars + 1, np.int32)
            inner = np.zeros(int(nnz[0]), np.int32)
            self._check(self.L.tad_hessian_pattern(self.h, outer.ctypes.data_as(_ip), inner.ctypes.data_as(_ip)))
            self._pattern = (outer, inner)
        return self._pattern

    def _csr(self, vals):
        import scipy.sparse as sp
        outer, inner = self.hessian_pattern()
        return sp.csr_matrix((vals, inner, outer), shape=(self.n_vars, self.n_vars))

    # ---- data marshalling (ScalarFunctionImpl.hh:216-254) --------------------
    def x_from_data(self, read):
        x = np.full(self.n_vars, np.nan)
        for v in range(self.n_handles):
            x[v * self.var_dim:(v + 1) * self.var_dim] = read(v)
        if not np.all(np.isfinite(x)):
            raise TinyADError(TAD_ERR_NONFINITE, "Assertion failed: Not finite x")
        return x

    def x_to_data(self, x, write):
        x = _f64(x)
        if x.size != self.n_vars:
            raise TinyADError(TAD_ERR_ARG, "Assertion failed: x.size() == n_vars")
        for v in range(self.n_handles):
            write(v, x[v * self.var_dim:(v + 1) * self.var_dim])

    # ---- evaluation --------------------------------------------------------
    def _x(self, x) -> np.ndarray:
        x = _f64(x)
        if x.size != self.n_vars:
            raise TinyADError(TAD_ERR_ARG, f"Assertion failed: {x.size} == {self.n_vars}")
        return x

    def eval(self, x) -> float:
        x = self._x(x)
        f = np.zeros(1)
        self._check(self.L.tad_eval(self.h, _d(x), _d(f)))
        return float(f[0])

    __call__ = eval

    def eval_with_gradient(self, x):
        x = self._x(x)
        f = np.zeros(1)
        g = np.zeros(self.n_vars)
        self._check(self.L.tad_eval_with_gradient(self.h, _d(x), _d(f), _d(g)))
        return float(f[0]), g

    def eval_with_derivatives(self, x):
        x = self._x(x)
        f = np.zeros(1)
        g = np.zeros(self.n_vars)
        outer, inner = self.hessian_pattern()
        vals = np.zeros(inner.size)
        self._check(self.L.tad_eval_with_derivatives(self.h, _d(x), _d(f), _d(g), _d(vals)))
        return float(f[0]), g, self._csr(vals)

    def eval_hessian(self, x):
        return self.eval_with_derivatives(x)[2]

    def eval_hessian_of_quadratic(self):
        return self.eval_hessian(np.zeros(self.n_vars))

    def eval_with_hessian_proj(self, x, projection_eps: float = default_hessian_projection_eps):
        x = self._x(x)
        f = np.zeros(1)
        g = np.zeros(self.n_vars)
        outer, inner = self.hessian_pattern()
        vals = np.zeros(inner.size)
        self._check(self.L.tad_eval_with_hessian_proj(self.h, _d(x), projection_eps, _d(f), _d(g), _d(vals)))
        return float(f[0]), g, self._csr(vals)

    # ---- solver utilities ----------------------------------------------------
    def newton_direction(self, x, projection_eps: float = default_hessian_projection_eps, projected: bool = True,
                         w_identity: float = 0.0):
        """d = -(H(x) + w I)^-1 g(x) (device PCG; NewtonDirection.hh:25-48), H
        projected (default) or exact.  Returns (d, f, g)."""
        x = self._x(x)
        d = np.zeros(self.n_vars)
        g = np.zeros(self.n_vars)
        f = np.zeros(1)
        self._check(self.L.tad_newton_direction(self.h, _d(x), int(projected), projection_eps, float(w_identity), _d(d),
                                                _d(f), _d(g)),
                    allow=(TAD_ERR_PCG_NOCONV,))
        return d, float(f[0]), g

    def newton_decrement(self, d, g) -> float:
        """newton_decrement(d, g) = -d.g / 2 (NewtonDecrement.hh:20-26), reduced
        on the device in a fixed order."""
        d, g = self._x(d), self._x(g)
        out = np.zeros(1)
        self._check(self.L.tad_newton_decrement(self.h, _d(d), _d(g), _d(out)))
        return float(out[0])

    def newton_decrement_device(self, d_ptr: int, g_ptr: int) -> float:
        """newton_decrement on device-resident d and g (pointers to n_vars doubles)."""
        out = np.zeros(1)
        self._check(self.L.tad_newton_decrement_d(self.h, ctypes.c_void_p(d_ptr), ctypes.c_void_p(g_ptr), _d(out)))
        return float(out[0])

    def newton_direction_reduced_basis(self, x, B, projection_eps: float = default_hessian_projection_eps,
                                       w_identity: float = 0.0):
        """newton_direction_reduced_basis(g, H_proj, B, solver, w): d = B (B^T H B
        + w I)^-1 (-B^T g) with g, H_proj at x and B an (n_vars x m) scipy
        sparse basis.  Returns (d, f, g)."""
        import scipy.sparse as sp
        x = self._x(x)
        Bc = sp.csr_matrix(B)
        if Bc.shape[0] != self.n_vars:
            raise ValueError(f"basis has {Bc.shape[0]} rows, the problem {self.n_vars} variables")
        Bc.sort_indices()
        outer = np.ascontiguousarray(Bc.indptr, dtype=np.int32)
        inner = np.ascontiguousarray(Bc.indices, dtype=np.int32)
        vals = np.ascontiguousarray(Bc.data, dtype=np.float64)
        d = np.zeros(self.n_vars)
        g = np.zeros(self.n_vars)
        f = np.zeros(1)
        self._check(self.L.tad_newton_direction_reduced_basis(self.h, _d(x), int(Bc.shape[1]),
                                                              outer.ctypes.data_as(_ip), inner.ctypes.data_as(_ip),
                                                              _d(vals), projection_eps, w_identity, _d(d), _d(f), _d(g)),
                    allow=(TAD_ERR_PCG_NOCONV,))
        return d, float(f[0]), g

    def line_search(self, x0, d, f, g, s_max: float = 1.0):
        """line_search(x0, d, f, g, func, s_max) -> x (x0 when no decrease)."""
        x0, d, g = self._x(x0), self._x(d), self._x(g)
        xo = np.zeros(self.n_vars)
        fo = np.zeros(1)
        self._check(self.L.tad_line_search(self.h, _d(x0), _d(d), float(f), _d(g), s_max, _d(xo), _d(fo)),
                    allow=(TAD_ERR_LS_FAIL,))
        return xo

    def newton_solve(self, x, n_iters: int, projection_eps: float = default_hessian_projection_eps,
                     stop_decrement: float = 0.0):
        """n_iters Projected-Newton iterations on the device.  Returns (x, f_hist)."""
        x = self._x(x).copy()
        fh = np.zeros(n_iters + 1)
        done = ctypes.c_int(0)
        self._check(self.L.tad_newton_solve(self.h, _d(x), n_iters, projection_eps, stop_decrement, _d(fh),
                                            ctypes.byref(done)))
        return x, fh[:done.value + 1]

    def newton_solve_inplace(self, x: np.ndarray, n_iters: int,
                             projection_eps: float = default_hessian_projection_eps, stop_decrement: float = 0.0):
        """Like newton_solve, updating the caller's float64 host array in place
        (no extra copies; pass pinned memory for fast transfers)."""
        if x.dtype != np.float64 or not x.flags["C_CONTIGUOUS"] or x.size != self.n_vars:
            raise TinyADError(TAD_ERR_ARG, "x must be a contiguous float64 array of n_vars entries")
        fh = np.zeros(n_iters + 1)
        done = ctypes.c_int(0)
        self._check(self.L.tad_newton_solve(self.h, _d(x), n_iters, projection_eps, stop_decrement, _d(fh),
                                            ctypes.byref(done)))
        return fh[:done.value + 1]

    @property
    def stream_ptr(self) -> int:
        s = ctypes.c_void_p()
        self._check(self.L.tad_get_stream(self.h, ctypes.byref(s)))
        return int(s.value or 0)

    def newton_solve_device(self, x_ptr: int, n_iters: int, projection_eps: float = default_hessian_projection_eps,
                            stop_decrement: float = 0.0):
        """Newton iterations on a device-resident x (pointer to n_vars doubles)."""
        fh = np.zeros(n_iters + 1)
        done = ctypes.c_int(0)
        self._check(self.L.tad_newton_solve_d(self.h, ctypes.c_void_p(x_ptr), n_iters, projection_eps, stop_decrement,
                                              _d(fh), ctypes.byref(done)))
        return fh[:done.value + 1]

    def adjoint_rest_gradient(self, x, dLdx, rest, projected: bool = True,
                              projection_eps: float = default_hessian_projection_eps):
        """dL/d(rest positions) at a minimiser x for dL/dx given (adjoint
        solve + mixed second derivatives).  Returns (dL/drest (n_handles, 3),
        lambda, pcg_iters)."""
        x, dLdx = self._x(x), self._x(dLdx)
        rest = _f64(rest).reshape(-1)
        if rest.size != 3 * self.n_handles:
            raise TinyADError(TAD_ERR_ARG, "rest must hold n_handles x 3 positions")
        out = np.zeros(3 * self.n_handles)
        lam = np.zeros(self.n_vars)
        it = ctypes.c_int(0)
        self._check(self.L.tad_adjoint_rest_gradient(self.h, _d(x), _d(dLdx), _d(rest), int(projected), projection_eps,
                                                     _d(out), _d(lam), ctypes.byref(it)), allow=(TAD_ERR_PCG_NOCONV,))
        return out.reshape(-1, 3), lam, it.value

    @property
    def launch_count(self) -> int:
        n = np.zeros(1, np.int64)
        self._check(self.L.tad_launch_count(self.h, n.ctypes.data_as(_i64p)))
        return int(n[0])

    def profile_kernels(self, x_ptr: int, reps: int = 5) -> dict:
        """Per-launch ms of the main kernels at device x (CUDA events)."""
        ms = np.zeros(5)
        self._check(self.L.tad_profile_kernels(self.h, ctypes.c_void_p(x_ptr), reps, _d(ms)))
        return {"elem_hessian": ms[0], "assemble": ms[1], "spmv": ms[2], "pcg_update": ms[3], "ls_energy": ms[4]}

    def last_solve_stats(self) -> dict:
        ms = np.zeros(4)
        it = np.zeros(1, np.int64)
        tr = np.zeros(1, np.int64)
        self._check(self.L.tad_last_solve_stats(self.h, _d(ms), it.ctypes.data_as(_i64p), tr.ctypes.data_as(_i64p)))
        return {"ms_eval": ms[0], "ms_assemble": ms[1], "ms_pcg": ms[2], "ms_linesearch": ms[3],
                "pcg_iters": int(it[0]), "ls_trials": int(tr[0])}


def debug_scalar_op(op: int, a, b=(0.0, 0.0, 0.0), precision: int = PREC_FP64) -> np.ndarray:
    """Apply one device Scalar<1> operator (op codes in include/tad.h)."""
    L = load()
    a3, b3, out = _f64(a), _f64(b), np.zeros(3)
    rc = L.tad_debug_scalar_op(op, precision, _d(a3), _d(b3), _d(out))
    if rc != TAD_OK:
        raise TinyADError(rc, L.tad_last_error_message().decode())
    return out


def solve_minimiser(w, x0, newton_iters: int = 30, full_steps: int = 2, tol: float = 1e-13, max_iters: int = 20000):
    """x* = argmin E(x) for workload w from x0 on the device: Projected-Newton
    iterations, then full Newton steps on the exact Hessian (quadratic
    convergence to the minimiser the adjoint differentiates).  Returns
    (x*, the ScalarFunction)."""
    fn = ScalarFunction.from_workload(w, pcg_rel_tol=tol, pcg_max_iters=max_iters)
    x, _ = fn.newton_solve(x0, newton_iters)
    for _ in range(full_steps):
        d, f, g = fn.newton_direction(x, projected=False)
        x = x + d
    return x, fn


class VectorFunction(ScalarFunction):
    """A vector function r: R^n -> R^m defined by per-element residual functors.

    Mirrors TinyAD::VectorFunction<d, double, Eigen::Index>
    (include/TinyAD/VectorFunction.hh) for the built-in residual functors
    (tad_vector_energy in include/tad.h); user functors use the C++ front end.
    The inherited scalar methods act on the sum of squares f = |r|^2
    (eval = eval_sum_of_squares, eval_with_gradient gives g = 2 J^T r,
    newton_solve runs Gauss-Newton with the Armijo line search on f).
    """

    def add_elements(self, energy: int, handles, params, n_outputs: int):
        """add_elements<N, M>(range, lambda) for a built-in residual functor."""
        handles = np.ascontiguousarray(handles, dtype=np.int32)
        if handles.ndim == 1:
            handles = handles[:, None]
        params = _f64(params)
        if params.ndim == 1:
            params = params[:, None]
        n, N = handles.shape
        self._check(self.L.tad_add_vector_elements(self.h, int(energy), N, int(n_outputs), n, handles.ctypes.data_as(_ip),
                                                   _d(params), params.shape[1] if n > 0 else int(params.shape[-1])))
        self._jpattern = None

    @property
    def n_outputs(self) -> int:
        return int(self.L.tad_n_outputs(self.h))

    def _jacobian_pattern(self):
        if getattr(self, "_jpattern", None) is None:
            nnz = np.zeros(1, np.int64)
            self._check(self.L.tad_vec_jacobian_nnz(self.h, nnz.ctypes.data_as(_i64p)))
            m = self.n_outputs
            outer = np.zeros(m + 1, np.int32)
            inner = np.zeros(int(nnz[0]), np.int32)
            self._check(self.L.tad_vec_jacobian_pattern(self.h, outer.ctypes.data_as(_ip), inner.ctypes.data_as(_ip)))
            self._jpattern = (outer, inner)
        return self._jpattern

    def _jacobian(self, values):
        import scipy.sparse as sp
        outer, inner = self._jacobian_pattern()
        return sp.csr_matrix((values, inner, outer), shape=(self.n_outputs, self.n_vars))

    def eval_vector(self, x) -> np.ndarray:
        """VectorFunction::eval(x): the residual vector r."""
        x = self._x(x)
        r = np.zeros(self.n_outputs)
        self._check(self.L.tad_vec_eval(self.h, _d(x), _d(r)))
        return r

    def eval_sum_of_squares(self, x) -> float:
        return self.eval(x)

    def eval_with_jacobian(self, x):
        """(r, J), J the n_outputs x n_vars Jacobian (scipy CSR)."""
        x = self._x(x)
        outer, inner = self._jacobian_pattern()
        r = np.zeros(self.n_outputs)
        vals = np.zeros(inner.size)
        self._check(self.L.tad_vec_eval_with_jacobian(self.h, _d(x), _d(r), _d(vals)))
        return r, self._jacobian(vals)

    def eval_with_derivatives(self, x):
        """(r, J, [H_i]): the residual Hessians as a list of n_vars x n_vars
        scipy CSR matrices, one per residual."""
        import scipy.sparse as sp
        x = self._x(x)
        outer, inner = self._jacobian_pattern()
        m = self.n_outputs
        nnz = np.zeros(1, np.int64)
        self._check(self.L.tad_vec_hessians_nnz(self.h, nnz.ctypes.data_as(_i64p)))
        r = np.zeros(m)
        vals = np.zeros(inner.size)
        hp = np.zeros(m + 1, np.int64)
        hr = np.zeros(int(nnz[0]), np.int32)
        hc = np.zeros(int(nnz[0]), np.int32)
        hv = np.zeros(int(nnz[0]))
        self._check(self.L.tad_vec_eval_with_derivatives(self.h, _d(x), _d(r), _d(vals), hp.ctypes.data_as(_i64p),
                                                         hr.ctypes.data_as(_ip), hc.ctypes.data_as(_ip), _d(hv)))
        H = [sp.csr_matrix((hv[hp[i]:hp[i + 1]], (hr[hp[i]:hp[i + 1]], hc[hp[i]:hp[i + 1]])),
                           shape=(self.n_vars, self.n_vars)) for i in range(m)]
        return r, self._jacobian(vals), H

    def eval_sum_of_squares_with_derivatives(self, x):
        """(f, g, r, J) with f = |r|^2, g = 2 J^T r."""
        x = self._x(x)
        outer, inner = self._jacobian_pattern()
        f = np.zeros(1)
        g = np.zeros(self.n_vars)
        r = np.zeros(self.n_outputs)
        vals = np.zeros(inner.size)
        self._check(self.L.tad_eval_sum_of_squares_with_derivatives(self.h, _d(x), _d(f), _d(g), _d(r), _d(vals)))
        return float(f[0]), g, r, self._jacobian(vals)

    def gauss_newton_direction(self, x, w_identity: float = 0.0):
        """gauss_newton_direction(r, J, solver, w) at x: d = -(J^T J + w I)^-1 J^T r.
        Returns (d, f, g)."""
        x = self._x(x)
        d = np.zeros(self.n_vars)
        g = np.zeros(self.n_vars)
        f = np.zeros(1)
        self._check(self.L.tad_gauss_newton_direction(self.h, _d(x), float(w_identity), _d(d), _d(f), _d(g)),
                    allow=(TAD_ERR_PCG_NOCONV,))
        return d, float(f[0]), g


class Batch:
    """Many independent meshes solved together (tad_batch_* in include/tad.h).

    workloads: list of meshes.Workload with the same var_dim and term energies
    (one term per energy, in the same order)."""

    def __init__(self, workloads, settings: Settings | None = None, **kw):
        self.L = load()
        self.ws = workloads
        self.var_dim = workloads[0].var_dim
        self.n_meshes = len(workloads)
        self.settings = settings if settings is not None else default_settings(**kw)
        nh = np.array([w.n_handles for w in workloads], np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(nh)]) * self.var_dim
        self.n_vars = int(self.offsets[-1])
        h = ctypes.c_void_p()
        self._check(self.L.tad_batch_create(self.var_dim, self.n_meshes, nh.ctypes.data_as(_i64p),
                                            ctypes.byref(self.settings), ctypes.byref(h)))
        self.h = h
        for t in range(len(workloads[0].terms)):
            terms = [w.terms[t] for w in workloads]
            cnt = np.array([tt.handles.shape[0] for tt in terms], np.int64)
            handles = np.ascontiguousarray(np.concatenate([tt.handles for tt in terms]), np.int32)
            params = np.ascontiguousarray(np.concatenate([tt.params for tt in terms]))
            self._check(self.L.tad_batch_add_elements(self.h, terms[0].energy, terms[0].valence,
                                                      cnt.ctypes.data_as(_i64p), handles.ctypes.data_as(_ip),
                                                      _d(params), params.shape[1]))

    def _check(self, rc, allow=()):
        if rc != TAD_OK and rc not in allow:
            raise TinyADError(rc, self.L.tad_last_error_message().decode())
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.L.tad_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def x0(self) -> np.ndarray:
        return np.concatenate([w.x0 for w in self.ws])

    def split(self, x):
        return [x[self.offsets[m]:self.offsets[m + 1]] for m in range(self.n_meshes)]

    def newton_solve(self, x, n_iters: int, projection_eps: float = default_hessian_projection_eps):
        x = _f64(x).copy()
        fh = np.zeros((n_iters + 1, self.n_meshes))
        self._check(self.L.tad_batch_newton_solve(self.h, _d(x), n_iters, projection_eps, _d(fh)))
        return x, fh

    def newton_solve_device(self, x_ptr: int, n_iters: int, projection_eps: float = default_hessian_projection_eps,
                            history: bool = False):
        fh = np.zeros((n_iters + 1, self.n_meshes)) if history else None
        self._check(self.L.tad_batch_newton_solve_d(self.h, ctypes.c_void_p(x_ptr), n_iters, projection_eps,
                                                    _d(fh) if history else None))
        return fh

    def autotune(self, x_ptr: int, projection_eps: float = default_hessian_projection_eps) -> dict:
        out = np.zeros(3)
        self._check(self.L.tad_batch_autotune(self.h, ctypes.c_void_p(x_ptr), projection_eps, _d(out)))
        return {"chunk_rows": int(out[0]), "threads": int(out[1]), "ms_per_iteration": float(out[2])}

    def set_chunking(self, chunk_rows: int, threads: int):
        self._check(self.L.tad_batch_set_chunking(self.h, chunk_rows, threads))

    @property
    def stream_ptr(self) -> int:
        p = ctypes.c_void_p()
        self._check(self.L.tad_batch_problem(self.h, ctypes.byref(p)))
        s = ctypes.c_void_p()
        self._check(self.L.tad_get_stream(p, ctypes.byref(s)))
        return int(s.value or 0)


def measure_fma_peak(precision: int) -> float:
    """CUDA-core FMA throughput (TFLOP/s) measured on the current GPU."""
    L = load()
    out = np.zeros(1)
    rc = L.tad_measure_fma_peak(precision, _d(out))
    if rc != TAD_OK:
        raise TinyADError(rc, L.tad_last_error_message().decode())
    return float(out[0])


def scalar_function(var_dim: int, n_handles: int, **kw) -> ScalarFunction:
    """scalar_function<d>(range(n)) (ScalarFunctionImpl.hh:418-442)."""
    return ScalarFunction(var_dim, n_handles, **kw)
