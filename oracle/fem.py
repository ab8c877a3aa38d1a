"""Per-mesh operators of the FEM path, FP64 restatement.

Each function cites the simkit routine whose result it reproduces.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sps


def shape_gradients(X: np.ndarray, T: np.ndarray) -> np.ndarray:
    """Rest-shape barycentric gradients per simplex, shape (t, d+1, d).

    Row ``a`` is grad N_a, so that ``F = sum_a x_a (x) grad N_a``.  This is the
    transpose of simkit's per-element ``D = (H (X^T H)^-1)^T``
    (``simkit/deformation_jacobian.py:43-61``, ``deformation_gradient.py:48-62``).
    """
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T)
    d = X.shape[1]
    E = (X[T[:, 1:]] - X[T[:, [0]]]).transpose(0, 2, 1)   # columns: edges from corner 0
    Einv = np.linalg.inv(E)                                  # (t, d, d); row j = grad N_{j+1}
    G = np.empty((T.shape[0], d + 1, d))
    G[:, 1:, :] = Einv
    G[:, 0, :] = -Einv.sum(axis=1)
    return G


def deformation_gradient(X, T, U) -> np.ndarray:
    """F per element from rest X and deformed U.  Reference: ``deformation_gradient.py:8-67``."""
    G = shape_gradients(X, T)
    return np.einsum("tai,taj->tij", np.asarray(U, dtype=np.float64)[T], G)


def deformation_jacobian(X, T) -> sps.csc_matrix:
    """Sparse J with ``(J x)[d*d*e + d*i + j] = F_e[i, j]``.

    Reference: ``simkit/deformation_jacobian.py:9-87``.  Exact zeros are
    dropped, as scipy's sparse product at :86 drops them.
    """
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T)
    t, k = T.shape
    d = X.shape[1]
    G = shape_gradients(X, T)                                   # (t, k, d)
    e = np.arange(t)[:, None, None, None]
    i = np.arange(d)[None, :, None, None]
    j = np.arange(d)[None, None, :, None]
    a = np.arange(k)[None, None, None, :]
    rows = np.broadcast_to(d * d * e + d * i + j, (t, d, d, k))
    cols = np.broadcast_to(d * T[:, None, None, :] + i, (t, d, d, k))
    vals = np.broadcast_to(G.transpose(0, 2, 1)[:, None, :, :], (t, d, d, k))  # G[e, a, j]
    del a
    J = sps.csc_matrix((vals.ravel(), (rows.ravel(), cols.ravel())),
                       shape=(t * d * d, X.shape[0] * d))
    J.eliminate_zeros()
    return J


def tet_volumes(X, T) -> np.ndarray:
    """Signed det([e1 e2 e3]) / 6.  Reference: ``tetrahedron_volumes.py:26-27``, ``volume.py:14-41``."""
    X = np.asarray(X, dtype=np.float64)
    e = X[T[:, 1:]] - X[T[:, [0]]]
    return (np.linalg.det(e) / 6.0).reshape(-1, 1)


def lumped_mass(X, T, rho) -> np.ndarray:
    """Per-vertex lumped mass sum_{e ∋ v} rho_e vol_e / (d+1).  Reference: ``massmatrix.py:40-50``."""
    vol = tet_volumes(X, T).ravel()
    m_e = vol * np.broadcast_to(np.asarray(rho, dtype=np.float64).ravel(), vol.shape)
    m = np.zeros(X.shape[0])
    np.add.at(m, np.asarray(T).ravel(), np.repeat(m_e / T.shape[1], T.shape[1]))
    return m


def gravity_force(X, T, a=-9.8, rho=1.0, direction=(0.0, 1.0, 0.0)) -> np.ndarray:
    """M (a * direction) per vertex, (n, 3).  Reference: ``gravity_force.py:35-42`` (axis 1 there)."""
    m = lumped_mass(X, T, rho)
    return m[:, None] * (a * np.asarray(direction, dtype=np.float64))[None, :]


def ympr_to_lame(ym, pr):
    """Reference: ``ympr_to_lame.py:32-34``."""
    mu = ym / (2.0 * (1.0 + pr))
    lam = ym * pr / ((1.0 + pr) * (1.0 - 2.0 * pr))
    return mu, lam


def selection_matrix(idx, n: int) -> sps.csc_matrix:
    """Row selector ``G x = x[idx]``.  Reference: ``selection_matrix.py:26-35``."""
    idx = np.asarray(idx).ravel()
    return sps.csc_matrix((np.ones(idx.size), (np.arange(idx.size), idx)), shape=(idx.size, n))
