"""Synthetic cantilever beams: the workloads the solver is measured on.

A beam is a regular grid of ``nx x ny x nz`` cubes of side ``cell``, each cube
split into six tetrahedra around its (0,0,0)-(1,1,1) diagonal (Kuhn split),
all positively oriented.  Vertices on the ``x = 0`` face are pinned.  The
arrays match simkit's conventions: ``X`` is (n, 3) float64, ``T`` is (t, 4),
``mu``/``lam`` are (t, 1) (``simkit/ympr_to_lame.py:32-34``), and gravity is
the lumped mass times the acceleration (``simkit/gravity_force.py:35-42``,
generalised to any direction).

Sizes of the three standard workloads:

* 8 x 8 x 32 cubes (length along x):       12,288 tets, 2,673 vertices
* 32 x 32 x 128 cubes, jittered rest shape: 786,432 tets, 140,481 vertices
* 512 beams, ny, nx in {4..16}, nz in {8..48}, random material and gravity
"""

from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np

# The six monotone lattice paths from corner (0,0,0) to (1,1,1).
_PERMS = list(itertools.permutations(range(3)))


def _perm_sign(p) -> int:
    s = 1
    p = list(p)
    for i in range(3):
        for j in range(i + 1, 3):
            if p[i] > p[j]:
                s = -s
    return s


def beam_mesh(nx: int, ny: int, nz: int, cell: float = 0.025):
    """Rest positions (n, 3) and tets (t, 4) of an nx x ny x nz Kuhn-split grid.

    Vertex (i, j, k) has index ``(i (ny+1) + j) (nz+1) + k``; cube (i, j, k)
    contributes tets ``6 ((i ny + j) nz + k) + p`` for the six paths p.
    """
    gi, gj, gk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    X = np.stack([gi, gj, gk], axis=-1).reshape(-1, 3).astype(np.float64) * cell

    def vid(i, j, k):
        return (i * (ny + 1) + j) * (nz + 1) + k

    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    tets = np.empty((ci.size, 6, 4), dtype=np.int64)
    for p_idx, p in enumerate(_PERMS):
        path = [np.zeros(3, dtype=np.int64)]
        for ax in p:
            step = path[-1].copy()
            step[ax] += 1
            path.append(step)
        corners = [vid(ci + s[0], cj + s[1], ck + s[2]) for s in path]
        if _perm_sign(p) < 0:
            corners[1], corners[2] = corners[2], corners[1]
        tets[:, p_idx, :] = np.stack(corners, axis=-1)
    return X, tets.reshape(-1, 4)


def beam_meshes(dims, cell: float = 0.025):
    """Rest positions and tets of several Kuhn-split beams, concatenated.

    ``dims`` is a sequence of (nx, ny, nz).  Returns (X, T, v_off, t_off): beam s
    owns vertices [v_off[s], v_off[s+1]) and tets [t_off[s], t_off[s+1]), and
    its slices equal ``beam_mesh(*dims[s], cell)`` with tets offset by v_off[s].
    All shapes are generated together with integer array arithmetic.
    """
    d = np.asarray(dims, dtype=np.int64).reshape(-1, 3)
    S = d.shape[0]
    nx, ny, nz = d[:, 0], d[:, 1], d[:, 2]
    nv = (nx + 1) * (ny + 1) * (nz + 1)
    nc = nx * ny * nz
    v_off = np.concatenate([[0], np.cumsum(nv)])
    c_off = np.concatenate([[0], np.cumsum(nc)])
    sv = np.repeat(np.arange(S), nv)
    lv = np.arange(v_off[-1]) - v_off[sv]
    NY, NZ = ny[sv] + 1, nz[sv] + 1
    X = np.stack([lv // (NY * NZ), (lv // NZ) % NY, lv % NZ], axis=-1).astype(np.float64) * cell
    sc = np.repeat(np.arange(S), nc)
    lc = np.arange(c_off[-1]) - c_off[sc]
    cy, cz = ny[sc], nz[sc]
    ci, cj, ck = lc // (cy * cz), (lc // cz) % cy, lc % cz
    VY, VZ, base = cy + 1, cz + 1, v_off[sc]

    def vid(i, j, k):
        return (i * VY + j) * VZ + k + base

    T = np.empty((lc.size, 6, 4), dtype=np.int64)
    for p_idx, p in enumerate(_PERMS):
        step = np.zeros(3, dtype=np.int64)
        corners = [vid(ci, cj, ck)]
        for ax in p:
            step[ax] += 1
            corners.append(vid(ci + step[0], cj + step[1], ck + step[2]))
        if _perm_sign(p) < 0:
            corners[1], corners[2] = corners[2], corners[1]
        T[:, p_idx, :] = np.stack(corners, axis=-1)
    return X, T.reshape(-1, 4), v_off, 6 * c_off


@dataclass
class BeamSpec:
    """One beam instance: rest mesh, material, loading and pins (FP64 host arrays)."""
    X: np.ndarray                 # (n, 3) rest positions
    T: np.ndarray                 # (t, 4) tets
    mu: np.ndarray                # (t, 1)
    lam: np.ndarray               # (t, 1)
    rho: float                    # density
    gravity: np.ndarray           # (3,) acceleration vector, m/s^2
    pinned: np.ndarray            # (p,) pinned vertex indices
    dims: tuple = (0, 0, 0)
    ym: np.ndarray = field(default=None)   # (t,) Young's modulus
    pr: np.ndarray = field(default=None)   # (t,) Poisson ratio

    @property
    def n_verts(self) -> int:
        return self.X.shape[0]

    @property
    def n_tets(self) -> int:
        return self.T.shape[0]


def _lame(ym, pr):
    mu = ym / (2.0 * (1.0 + pr))
    lam = ym * pr / ((1.0 + pr) * (1.0 - 2.0 * pr))
    return mu, lam


def make_beam(nx, ny, nz, cell=0.025, ym=1e6, pr=0.45, rho=1000.0,
              gravity=(0.0, -9.8, 0.0), jitter=0.0, seed=0) -> BeamSpec:
    """A beam with per-tet Young's modulus ``ym`` (scalar or (t,)) and ratio ``pr``."""
    X, T = beam_mesh(nx, ny, nz, cell)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        J = rng.uniform(-jitter, jitter, size=X.shape) * cell
        J[X[:, 0] == 0.0, 0] = 0.0           # the pinned face stays planar
        X = X + J
    t = T.shape[0]
    ym = np.broadcast_to(np.asarray(ym, dtype=np.float64), (t,)).copy()
    pr = np.broadcast_to(np.asarray(pr, dtype=np.float64), (t,)).copy()
    mu, lam = _lame(ym, pr)
    pinned = np.nonzero(np.arange(X.shape[0]) < (ny + 1) * (nz + 1))[0]
    return BeamSpec(X=X, T=T, mu=mu.reshape(-1, 1), lam=lam.reshape(-1, 1), rho=float(rho),
                    gravity=np.asarray(gravity, dtype=np.float64), pinned=pinned,
                    dims=(nx, ny, nz), ym=ym, pr=pr)


def beam_small_steady(nx=32, ny=8, nz=8) -> BeamSpec:
    """The 8 x 8 x 32 beam: E = 1e6 Pa, nu = 0.45, rho = 1000, gravity -y, x = 0 pinned."""
    return make_beam(nx, ny, nz, cell=0.025, ym=1e6, pr=0.45, rho=1000.0)


def beam_large_jittered(nx=128, ny=32, nz=32, seed=0) -> BeamSpec:
    """The 32 x 32 x 128 beam: rest shape jittered by U(-0.1, 0.1) cells, E log-uniform [1e5, 1e7]."""
    rng = np.random.default_rng(seed)
    t = 6 * nx * ny * nz
    ym = np.exp(rng.uniform(np.log(1e5), np.log(1e7), size=t))
    return make_beam(nx, ny, nz, cell=0.025, ym=ym, pr=0.45, rho=1000.0, jitter=0.1, seed=seed + 1)


def beam_batch(count=512, seed=0, ny_range=(4, 16), nz_range=(8, 48), nx_range=(4, 16)):
    """``count`` independent beams with seeded dims, material and gravity direction.

    Per instance: nx, ny uniform in {4..16}, nz uniform in {8..48}; Young's
    modulus log-uniform [1e5, 1e7] and Poisson ratio uniform [0.30, 0.49]
    (uniform over the instance); gravity 9.8 m/s^2 along a uniform direction
    on the unit sphere.
    """
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        nx = int(rng.integers(nx_range[0], nx_range[1] + 1))
        ny = int(rng.integers(ny_range[0], ny_range[1] + 1))
        nz = int(rng.integers(nz_range[0], nz_range[1] + 1))
        ym = float(np.exp(rng.uniform(np.log(1e5), np.log(1e7))))
        pr = float(rng.uniform(0.30, 0.49))
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        out.append(make_beam(nx, ny, nz, cell=0.025, ym=ym, pr=pr, rho=1000.0, gravity=9.8 * d))
    return out
