"""Linear (small-strain) elasticity element and assembled tiers, FP64 restatement.

Test infrastructure only: the checker of the GPU kernels, never the measured or
shipped path.

As simkit writes it in ``simkit/energies/linear_elasticity.py:43-136``::

    psi(F) = mu |eps|^2 + lam/2 tr(eps)^2,   eps = (F + F^T)/2 - I
    P(F)   = mu (F + F^T - 2 I) + lam tr(F - I) I
    H      = mu (I + T) + lam vec(I) vec(I)^T

with T the transposition of row-major vec(F).  The Hessian is constant and PSD;
simkit's ``linear_elasticity_hessian_x`` / ``_u`` (:199-230, :301-333) accept
``psd`` and ignore it, and so do the assembled tiers here.
"""

from __future__ import annotations

import numpy as np

from .snh import _F_of, _block_diag, _dim_of


def _batch(F):
    F = np.asarray(F, dtype=np.float64)
    d = F.shape[-1]
    return F.reshape(-1, d, d), d


def energy_element_F(F, mu, lam) -> np.ndarray:
    F, d = _batch(F)
    eps = 0.5 * (F + np.swapaxes(F, 1, 2)) - np.eye(d)[None]
    tr = np.trace(eps, axis1=1, axis2=2)
    return (np.asarray(mu, dtype=np.float64).reshape(-1) * np.sum(eps ** 2, axis=(1, 2))
            + 0.5 * np.asarray(lam, dtype=np.float64).reshape(-1) * tr ** 2).reshape(-1, 1)


def gradient_element_F(F, mu, lam) -> np.ndarray:
    F, d = _batch(F)
    I = np.eye(d)[None]
    mu = np.asarray(mu, dtype=np.float64).reshape(-1, 1, 1)
    lam = np.asarray(lam, dtype=np.float64).reshape(-1, 1, 1)
    tr = np.trace(F - I, axis1=1, axis2=2)[:, None, None]
    return mu * (F + np.swapaxes(F, 1, 2) - 2.0 * I) + lam * tr * I


def hessian_element_F(F, mu, lam) -> np.ndarray:
    F, d = _batch(F)
    n = d * d
    T = np.zeros((n, n))
    for i in range(d):
        for j in range(d):
            T[d * i + j, d * j + i] = 1.0
    vI = np.eye(d).reshape(-1)
    H1 = np.eye(n) + T
    H2 = np.outer(vI, vI)
    mu = np.asarray(mu, dtype=np.float64).reshape(-1, 1, 1)
    lam = np.asarray(lam, dtype=np.float64).reshape(-1, 1, 1)
    return np.broadcast_to(mu * H1[None] + lam * H2[None], (F.shape[0], n, n)).copy()


def energy_x(x, J, mu, lam, vol) -> float:
    F = _F_of(x, J, _dim_of(J, x))
    return float((np.asarray(vol).reshape(-1, 1) * energy_element_F(F, mu, lam)).sum())


def gradient_x(x, J, mu, lam, vol) -> np.ndarray:
    F = _F_of(x, J, _dim_of(J, x))
    P = gradient_element_F(F, mu, lam) * np.asarray(vol).reshape(-1, 1, 1)
    return J.T @ P.reshape(-1, 1)


def hessian_x(x, J, mu, lam, vol, psd: bool = True):
    """J^T blockdiag(vol He) J; ``psd`` has no effect (the Hessian is PSD)."""
    F = _F_of(x, J, _dim_of(J, x))
    He = hessian_element_F(F, mu, lam) * np.asarray(vol).reshape(-1, 1, 1)
    return (J.T @ _block_diag(He) @ J).tocsr()
