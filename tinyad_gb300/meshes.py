"""Seeded synthetic workloads for the sparse per-element derivative path.

The reference ships no large meshes (its fixtures are the tiny meshes of
tests/Meshes.hh); these generators build the workloads the benchmark and the
parity tests run on, identically for the CUDA path and the CPU oracle:

* ``disk_param(grid)``: planar parametrisation of a lifted, jittered disk.
  A grid x grid vertex lattice on [-1, 1]^2, split into triangles with
  alternating diagonals, clipped to the unit circle (triangles with all three
  vertices inside), reduced to its largest edge-connected manifold component;
  interior vertices jittered uniformly by +-0.2 h, lifted to
  z = 0.3 sin(3x) cos(2y).  Rest shape: each 3D triangle in its own
  orthonormal frame (Mr = [[l, e.f/l], [0, |e x f|/l]], weight = rest area).
  Initial UVs: Tutte embedding (uniform weights, boundary mapped to the unit
  circle by arc length).  Energy: symmetric Dirichlet per face, k = 6.
* ``tet_twist(cells)``: (cells+1)^3 lattice on [0, 1]^3, each cube split into
  6 tets along its main diagonal (Kuhn / Freudenthal), interior vertices
  jittered by +-0.1 h; symmetric Dirichlet per tet (k = 12) plus position
  penalties pinning the z=0 face to rest and pulling the z=1 face to its rest
  position twisted by 45 degrees about the vertical axis through (0.5, 0.5).
* ``planar_test_mesh()``: the 6-vertex / 4-face mesh with two position
  constraints of the reference's tests/Meshes.hh:12-42.

Everything is seeded (numpy PCG64) and deterministic.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI = 0
TAD_ENERGY_SYMMETRIC_DIRICHLET_TET = 1
TAD_ENERGY_POSITION_PENALTY = 2
TAD_ENERGY_QUADRATIC = 3
TAD_ENERGY_DIRICHLET_TRI = 4
# residual functors of vector terms (tad_vector_energy)
TAD_VEC_SYMMETRIC_DIRICHLET_TRI = 0
TAD_VEC_POSITION = 1


@dataclass
class Term:
    energy: int
    valence: int
    handles: np.ndarray          # (n_elem, valence) int32
    params: np.ndarray           # (n_elem, n_params) float64


@dataclass
class Workload:
    name: str
    var_dim: int
    n_handles: int
    x0: np.ndarray               # (n_handles * var_dim,) float64, interleaved
    terms: list = field(default_factory=list)
    rest: np.ndarray | None = None     # rest vertex positions (n_handles, 3)
    faces: np.ndarray | None = None
    info: dict = field(default_factory=dict)

    @property
    def n_vars(self) -> int:
        return self.var_dim * self.n_handles

    @property
    def n_elements(self) -> int:
        return sum(int(t.handles.shape[0]) for t in self.terms)


# ---------------------------------------------------------------------------
# triangle rest frames
# ---------------------------------------------------------------------------
def tri_rest_params(P: np.ndarray, F: np.ndarray) -> np.ndarray:
    """[Mr00 Mr10 Mr01 Mr11 w] per face from 3D rest positions P (column-major Mr)."""
    a, b, c = P[F[:, 0]], P[F[:, 1]], P[F[:, 2]]
    e = b - a
    f = c - a
    l = np.linalg.norm(e, axis=1)
    n = np.cross(e, f)
    an = np.linalg.norm(n, axis=1)
    out = np.zeros((F.shape[0], 5))
    out[:, 0] = l
    out[:, 1] = 0.0
    out[:, 2] = np.einsum("ij,ij->i", e, f) / l
    out[:, 3] = an / l
    out[:, 4] = 0.5 * an
    return out


# ---------------------------------------------------------------------------
# disk meshes
# ---------------------------------------------------------------------------
def _grid_disk_faces(grid: int):
    h = 2.0 / (grid - 1)
    ii, jj = np.meshgrid(np.arange(grid), np.arange(grid), indexing="ij")
    xy = np.stack([-1.0 + ii.ravel() * h, -1.0 + jj.ravel() * h], axis=1)
    vid = lambda i, j: i * grid + j  # noqa: E731
    ci, cj = np.meshgrid(np.arange(grid - 1), np.arange(grid - 1), indexing="ij")
    ci, cj = ci.ravel(), cj.ravel()
    v00, v10, v01, v11 = vid(ci, cj), vid(ci + 1, cj), vid(ci, cj + 1), vid(ci + 1, cj + 1)
    even = ((ci + cj) % 2) == 0
    t1 = np.where(even[:, None], np.stack([v00, v10, v11], 1), np.stack([v00, v10, v01], 1))
    t2 = np.where(even[:, None], np.stack([v00, v11, v01], 1), np.stack([v10, v11, v01], 1))
    F = np.concatenate([t1, t2], axis=0)
    inside = (xy[:, 0] ** 2 + xy[:, 1] ** 2) < 1.0
    F = F[inside[F].all(axis=1)]
    return xy, F, h


def _edge_components(F: np.ndarray) -> np.ndarray:
    """Label faces by connectivity through shared edges."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import connected_components

    nf = F.shape[0]
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]], 0)
    fid = np.concatenate([np.arange(nf)] * 3)
    key = np.minimum(e[:, 0], e[:, 1]).astype(np.int64) * (1 << 32) + np.maximum(e[:, 0], e[:, 1])
    order = np.argsort(key, kind="stable")
    ks, fs = key[order], fid[order]
    same = np.nonzero(ks[1:] == ks[:-1])[0]
    A = sp.coo_matrix((np.ones(same.size), (fs[same], fs[same + 1])), shape=(nf, nf))
    return connected_components(A, directed=False)[1]


def _boundary_edges(F: np.ndarray) -> np.ndarray:
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]], 0)
    key = np.minimum(e[:, 0], e[:, 1]).astype(np.int64) * (1 << 32) + np.maximum(e[:, 0], e[:, 1])
    uniq, inv, cnt = np.unique(key, return_inverse=True, return_counts=True)
    return e[cnt[inv] == 1]          # oriented as in their face (CCW)


def _clean_disk(F: np.ndarray) -> np.ndarray:
    """Largest edge-connected component with a single manifold boundary loop."""
    for _ in range(100):
        lab = _edge_components(F)
        vals, cnt = np.unique(lab, return_counts=True)
        F = F[lab == vals[np.argmax(cnt)]]
        be = _boundary_edges(F)
        deg = np.bincount(be.ravel())
        bad = np.nonzero(deg > 2)[0]
        if bad.size == 0:
            return F
        F = F[~np.isin(F, bad).any(axis=1)]
    raise RuntimeError("could not clean disk mesh")


def _boundary_loop(F: np.ndarray) -> np.ndarray:
    be = _boundary_edges(F)
    nxt = {int(a): int(b) for a, b in be}
    start = int(be[0, 0])
    loop = [start]
    v = nxt[start]
    while v != start:
        loop.append(v)
        v = nxt[v]
        if len(loop) > be.shape[0]:
            raise RuntimeError("boundary is not a single loop")
    if len(loop) != be.shape[0]:
        raise RuntimeError("boundary has several loops")
    return np.array(loop)


def tutte_embedding(P: np.ndarray, F: np.ndarray) -> np.ndarray:
    """Uniform-weight Tutte embedding of a disk onto the unit circle."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    nv = P.shape[0]
    loop = _boundary_loop(F)
    seg = np.linalg.norm(P[np.roll(loop, -1)] - P[loop], axis=1)
    t = np.concatenate([[0.0], np.cumsum(seg)[:-1]]) / seg.sum()
    uv = np.zeros((nv, 2))
    uv[loop, 0] = np.cos(2 * np.pi * t)
    uv[loop, 1] = np.sin(2 * np.pi * t)
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]], 0).astype(np.int64)
    key = np.unique(np.minimum(e[:, 0], e[:, 1]) * (1 << 32) + np.maximum(e[:, 0], e[:, 1]))
    e = np.stack([key >> 32, key & 0xFFFFFFFF], axis=1)
    A = sp.coo_matrix((np.ones(2 * len(e)), (np.r_[e[:, 0], e[:, 1]], np.r_[e[:, 1], e[:, 0]])), shape=(nv, nv)).tocsr()
    deg = np.asarray(A.sum(axis=1)).ravel()
    L = sp.diags(deg) - A
    is_b = np.zeros(nv, bool)
    is_b[loop] = True
    I = np.nonzero(~is_b)[0]
    B = np.nonzero(is_b)[0]
    LII = L[I][:, I].tocsc()
    rhs = -(L[I][:, B] @ uv[B])
    lu = spla.splu(LII, permc_spec="MMD_AT_PLUS_A")
    uv[I, 0] = lu.solve(np.ascontiguousarray(rhs[:, 0]))
    uv[I, 1] = lu.solve(np.ascontiguousarray(rhs[:, 1]))
    return uv


def disk_param(grid: int, seed: int = 0, jitter: float = 0.2, lift: bool = True,
               name: str | None = None) -> Workload:
    rng = np.random.default_rng(seed)
    xy, F, h = _grid_disk_faces(grid)
    F = _clean_disk(F)
    used = np.unique(F)
    remap = -np.ones(xy.shape[0], np.int64)
    remap[used] = np.arange(used.size)
    xy = xy[used]
    F = remap[F].astype(np.int32)
    nv = xy.shape[0]
    loop = _boundary_loop(F)
    interior = np.ones(nv, bool)
    interior[loop] = False
    xy = xy + interior[:, None] * rng.uniform(-jitter * h, jitter * h, size=(nv, 2))
    z = 0.3 * np.sin(3 * xy[:, 0]) * np.cos(2 * xy[:, 1]) if lift else np.zeros(nv)
    P = np.column_stack([xy, z])
    params = tri_rest_params(P, F)
    uv = tutte_embedding(P, F)
    w = Workload(name or f"disk{grid}", 2, nv, uv.reshape(-1).copy(),
                 [Term(TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI, 3, F.copy(), params)], rest=P, faces=F,
                 info={"grid": grid, "seed": seed, "n_faces": int(F.shape[0]), "n_verts": int(nv),
                       "boundary": loop})
    return w


def disk_param_pinned(grid: int, seed: int = 0, pin_weight: float = 10.0, name: str | None = None) -> Workload:
    """disk_param plus position penalties on two opposite boundary vertices
    (at their initial UVs), which remove the rigid-motion null space so the
    minimiser x*(rest) is unique -- the adjoint workload."""
    w = disk_param(grid, seed=seed, name=name or f"disk{grid}_pinned")
    loop = w.info["boundary"]
    pins = np.array([loop[0], loop[len(loop) // 2]], np.int32)
    uv = w.x0.reshape(-1, 2)
    pp = np.column_stack([uv[pins], np.full(2, pin_weight)])
    w.terms.append(Term(TAD_ENERGY_POSITION_PENALTY, 1, pins[:, None].copy(), pp))
    w.info["pins"] = pins
    return w


def with_rest(w: Workload, P: np.ndarray) -> Workload:
    """The same triangle workload with rest positions P (params recomputed)."""
    terms = []
    for t in w.terms:
        if t.energy == TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI:
            terms.append(Term(t.energy, t.valence, t.handles, tri_rest_params(P, t.handles)))
        else:
            terms.append(t)
    return Workload(w.name, w.var_dim, w.n_handles, w.x0.copy(), terms, rest=P, faces=w.faces, info=w.info)


# ---------------------------------------------------------------------------
# tet twist
# ---------------------------------------------------------------------------
def tet_rest_params(P: np.ndarray, T: np.ndarray) -> np.ndarray:
    a, b, c, d = (P[T[:, i]] for i in range(4))
    Mr = np.stack([b - a, c - a, d - a], axis=2)        # columns
    out = np.zeros((T.shape[0], 10))
    out[:, :9] = Mr.transpose(0, 2, 1).reshape(-1, 9)   # column-major flatten
    out[:, 9] = np.linalg.det(Mr) / 6.0
    return out


def tet_twist(cells: int, seed: int = 0, jitter: float = 0.1, angle_deg: float = 45.0,
              penalty_weight: float | None = None, name: str | None = None) -> Workload:
    rng = np.random.default_rng(seed)
    n = cells + 1
    h = 1.0 / cells
    ii, jj, kk = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    P = np.stack([ii.ravel() * h, jj.ravel() * h, kk.ravel() * h], axis=1)
    vid = lambda i, j, k: (i * n + j) * n + k  # noqa: E731
    interior = ((ii > 0) & (ii < cells) & (jj > 0) & (jj < cells) & (kk > 0) & (kk < cells)).ravel()
    P = P + interior[:, None] * rng.uniform(-jitter * h, jitter * h, size=P.shape)
    ci, cj, ck = (a.ravel() for a in np.meshgrid(np.arange(cells), np.arange(cells), np.arange(cells), indexing="ij"))
    unit = [np.array([1, 0, 0]), np.array([0, 1, 0]), np.array([0, 0, 1])]
    tets = []
    for perm in ([0, 1, 2], [0, 2, 1], [1, 0, 2], [1, 2, 0], [2, 0, 1], [2, 1, 0]):
        p0 = np.zeros(3, int)
        p1 = p0 + unit[perm[0]]
        p2 = p1 + unit[perm[1]]
        p3 = np.ones(3, int)
        vs = [vid(ci + p[0], cj + p[1], ck + p[2]) for p in (p0, p1, p2, p3)]
        tets.append(np.stack(vs, axis=1))
    T = np.concatenate(tets, 0)
    # orient positively
    a, b, c, d = (P[T[:, i]] for i in range(4))
    det = np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a)
    neg = det < 0
    T[neg, 1], T[neg, 2] = T[neg, 2].copy(), T[neg, 1].copy()
    T = T.astype(np.int32)
    params = tet_rest_params(P, T)
    bottom = np.nonzero(np.isclose(P[:, 2], 0.0))[0]
    top = np.nonzero(np.isclose(P[:, 2], 1.0))[0]
    th = math.radians(angle_deg)
    R = np.array([[math.cos(th), -math.sin(th)], [math.sin(th), math.cos(th)]])
    tgt_top = P[top].copy()
    tgt_top[:, :2] = (tgt_top[:, :2] - 0.5) @ R.T + 0.5
    cons = np.concatenate([bottom, top]).astype(np.int32)
    tgt = np.concatenate([P[bottom], tgt_top])
    if penalty_weight is None:
        penalty_weight = 100.0 / cons.size
    pp = np.column_stack([tgt, np.full(cons.size, penalty_weight)])
    terms = [Term(TAD_ENERGY_SYMMETRIC_DIRICHLET_TET, 4, T, params),
             Term(TAD_ENERGY_POSITION_PENALTY, 1, cons[:, None].copy(), pp)]
    return Workload(name or f"tet{cells}", 3, P.shape[0], P.reshape(-1).copy(), terms, rest=P, faces=T,
                    info={"cells": cells, "seed": seed, "n_tets": int(T.shape[0]), "n_verts": int(P.shape[0]),
                          "penalty_weight": penalty_weight, "angle_deg": angle_deg})


# ---------------------------------------------------------------------------
# the reference's planar test mesh (tests/Meshes.hh:12-42, NewtonTest.cc)
# ---------------------------------------------------------------------------
def planar_test_mesh() -> Workload:
    V_rest = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0], [0.0, 2.0], [1.0, 2.0]])
    V = V_rest.copy()
    V[:, 0] *= 0.5
    V[:, 1] *= 0.25
    F = np.array([[0, 1, 2], [1, 3, 2], [2, 3, 5], [2, 5, 4]], np.int32)
    Mr = np.stack([V_rest[F[:, 1]] - V_rest[F[:, 0]], V_rest[F[:, 2]] - V_rest[F[:, 0]]], axis=2)
    params = np.zeros((4, 5))
    params[:, :4] = Mr.transpose(0, 2, 1).reshape(-1, 4)
    params[:, 4] = 1.0 / F.shape[0]
    b = np.array([[0], [4]], np.int32)
    bc = np.array([[0.0, 0.0, 1.0], [-2.0, 0.0, 1.0]])
    terms = [Term(TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI, 3, F, params),
             Term(TAD_ENERGY_POSITION_PENALTY, 1, b, bc)]
    return Workload("planar_test_mesh", 2, 6, V.reshape(-1).copy(), terms, rest=np.column_stack([V_rest, np.zeros(6)]),
                    faces=F)


def disk_batch(n_meshes: int = 256, lo: int = 1000, hi: int = 50000, seed: int = 0) -> list:
    """Meshes with face counts drawn log-uniformly in [lo, hi]."""
    rng = np.random.default_rng(seed)
    targets = np.exp(rng.uniform(math.log(lo), math.log(hi), size=n_meshes))
    out = []
    for i, t in enumerate(targets):
        grid = max(8, int(round(1 + math.sqrt(2.0 * t / math.pi))))
        out.append(disk_param(grid, seed=seed * 100003 + i + 1, name=f"batch{i}"))
    return out


def residual_terms(w: Workload) -> list:
    """The residual form of a workload made of symmetric Dirichlet triangle
    and position penalty terms: (vector energy, handles, params, outputs) per
    term, with the same parameters, so that the sum of squares of the
    residuals equals the workload's energy (tests/GaussNewtonTest.cc:33-74)."""
    out = []
    for t in w.terms:
        if t.energy == TAD_ENERGY_SYMMETRIC_DIRICHLET_TRI:
            out.append((TAD_VEC_SYMMETRIC_DIRICHLET_TRI, t.handles, t.params, 8))
        elif t.energy == TAD_ENERGY_POSITION_PENALTY:
            out.append((TAD_VEC_POSITION, t.handles, t.params, w.var_dim))
        else:
            raise ValueError(f"no residual form for energy {t.energy}")
    return out
