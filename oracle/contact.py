"""Contact springs against a plane, FP64 restatement.

Test infrastructure only: the checker of the GPU kernels.

simkit ``simkit/energies/contact_springs_plane.py:44-200``: a vertex x_i with
(x_i - p) . n < 0 is in contact; the energy is k/2 sum_i m_i ((x_i - p) . n)^2
over contacting vertices (m the diagonal of M, identity by default), the
gradient k m_i ((x_i - p) . n) n and the Hessian block k m_i n n^T.  simkit
writes these with a selection matrix N of the contacting vertices' normals;
per vertex they are the same numbers.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sps


def _setup(X, p, n, M):
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    p = np.asarray(p, dtype=np.float64).reshape(-1)[:3]
    n = np.asarray(n, dtype=np.float64).reshape(3)
    m = np.ones(X.shape[0]) if M is None else np.asarray(M.diagonal() if sps.issparse(M) else np.diagonal(M))
    d = (X - p[None, :]) @ n
    return X, n, m, d, d < 0


def energy(X, k, p, n, M=None) -> float:
    """Reference: ``contact_springs_plane.py:44-86``."""
    X, n, m, d, under = _setup(X, p, n, M)
    return float((0.5 * k * m[under] * d[under] ** 2).sum())


def gradient(X, k, p, n, M=None) -> np.ndarray:
    """Reference: ``:87-130``."""
    X, n, m, d, under = _setup(X, p, n, M)
    g = np.zeros_like(X)
    g[under] = (k * m[under] * d[under])[:, None] * n[None, :]
    return g.reshape(-1, 1)


def hessian(X, k, p, n, M=None):
    """Reference: ``:131-200``."""
    X, n, m, d, under = _setup(X, p, n, M)
    nv = X.shape[0]
    blocks = np.zeros((nv, 3, 3))
    blocks[under] = (k * m[under])[:, None, None] * np.outer(n, n)[None]
    r = (3 * np.arange(nv)[:, None, None] + np.arange(3)[None, :, None]).repeat(3, axis=2)
    c = (3 * np.arange(nv)[:, None, None] + np.arange(3)[None, None, :]).repeat(3, axis=1)
    return sps.csc_matrix((blocks.ravel(), (r.ravel(), c.ravel())), shape=(3 * nv, 3 * nv))
