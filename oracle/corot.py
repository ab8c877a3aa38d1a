"""ARAP and fixed-corotated (FCR) element and assembled tiers, FP64 restatement.

Test infrastructure only: the checker of the GPU kernels, never the measured or
shipped path.

Both energies measure the distance of F from its rotation R = U V^T, where
U S V^T is the rotation-variant SVD (``simkit/svd_rv.py:8-52``: numpy's SVD,
then the last singular pair of U or V flipped so that det(U V^T) = +1, the
smallest singular value taking the sign)::

    ARAP  psi = mu/2 |F - R|^2                  (simkit/energies/arap.py:71-91)
          P   = mu (F - R)                      (:94-114)
          H   = mu (I - dR/dF)                  (:117-145)
    FCR   psi = mu |F - R|^2 + lam/2 (J - 1)^2  (simkit/energies/fcr.py:41-62)
          P   = 2 mu (F - R) + lam (J - 1) cof F                         (:65-125)
          H   = 2 mu (I - dR/dF) + lam c c^T + lam (J - 1) d2J/dF2        (:128-302)

with c = vec(cof F) row-major.  dR/dF is the closed form of
``simkit/rotation_gradient.py:12-70``: for each pair (i, j) of singular
directions, 2 / max(s_i + s_j, eps) t t^T with t = vec(U (e_i e_j^T - e_j e_i^T) V^T)/sqrt2
(eps = 1e-8 in 3D, 1e-12 in 2D, one pair in 2D).  simkit writes the FCR volume
terms entrywise from generated code; here they come from the determinant's
derivatives in ``oracle.snh``.  The assembled tiers weight by vol, optionally
PSD-project the weighted blocks and form J^T blockdiag(He) J (arap.py:242-325,
fcr.py:308-397), as for the neo-Hookean materials.
"""

from __future__ import annotations

import numpy as np

from .psd import psd_project
from .snh import _F_of, _block_diag, _dim_of, cofactor, det_hessian


def _batch(F, name):
    F = np.asarray(F, dtype=np.float64)
    d = F.shape[-1]
    if d not in (2, 3):
        raise ValueError(f"{name} supports dim=2 or dim=3")
    return F.reshape(-1, d, d), d


def _col(a):
    return np.asarray(a, dtype=np.float64).reshape(-1)


def svd_rv(F):
    """U, s (signed), V with F = U diag(s) V^T and det(U V^T) = +1.  Reference: ``svd_rv.py:8-52``."""
    F = np.asarray(F, dtype=np.float64)
    U, s, Vt = np.linalg.svd(F)
    V = np.swapaxes(Vt, -1, -2).copy()
    U = U.copy()
    s = s.copy()
    dU = np.linalg.det(U)
    dV = np.linalg.det(V)
    flip = dU * dV < 0          # det(U V^T) = -1: negate the last singular pair
    fu = flip & (dU < 0)
    fv = flip & (dV < 0)
    U[fu, :, -1] *= -1.0
    V[fv, :, -1] *= -1.0
    s[flip, -1] *= -1.0
    return U, s, V


def rotation(F):
    """R = U V^T of the rotation-variant SVD.  Reference: ``polar_svd.py:59-90``."""
    U, _, V = svd_rv(F)
    return U @ np.swapaxes(V, -1, -2)


_PAIRS = {2: ((0, 1),), 3: ((0, 1), (1, 2), (0, 2))}
_EPS = {2: 1e-12, 3: 1e-8}


def rotation_gradient_F(F):
    """dR/dF, (t, d*d, d*d) in row-major vec(F).  Reference: ``rotation_gradient.py:12-70``."""
    F, d = _batch(F, "rotation_gradient_F")
    U, s, V = svd_rv(F)
    K = np.zeros((F.shape[0], d * d, d * d))
    for i, j in _PAIRS[d]:
        T = (U[:, :, i, None] * V[:, None, :, j] - U[:, :, j, None] * V[:, None, :, i]) / np.sqrt(2.0)
        t = T.reshape(-1, d * d)
        w = 2.0 / np.maximum(s[:, i] + s[:, j], _EPS[d])
        K += w[:, None, None] * t[:, :, None] * t[:, None, :]
    return K


def _shear(F):
    return np.sum((F - rotation(F)) ** 2, axis=(1, 2))


def arap_energy_element_F(F, mu) -> np.ndarray:
    F, _ = _batch(F, "ARAP")
    return (0.5 * _col(mu) * _shear(F)).reshape(-1, 1)


def arap_gradient_element_F(F, mu) -> np.ndarray:
    F, _ = _batch(F, "ARAP")
    return _col(mu)[:, None, None] * (F - rotation(F))


def arap_hessian_element_F(F, mu) -> np.ndarray:
    F, d = _batch(F, "ARAP")
    return _col(mu)[:, None, None] * (np.eye(d * d)[None] - rotation_gradient_F(F))


def fcr_energy_element_F(F, mu, lam) -> np.ndarray:
    F, _ = _batch(F, "FCR")
    y = np.linalg.det(F) - 1.0
    return (_col(mu) * _shear(F) + 0.5 * _col(lam) * y * y).reshape(-1, 1)


def fcr_gradient_element_F(F, mu, lam) -> np.ndarray:
    F, _ = _batch(F, "FCR")
    y = np.linalg.det(F) - 1.0
    return (2.0 * _col(mu)[:, None, None] * (F - rotation(F))
            + (_col(lam) * y)[:, None, None] * cofactor(F))


def fcr_hessian_element_F(F, mu, lam) -> np.ndarray:
    F, d = _batch(F, "FCR")
    t = F.shape[0]
    lam = _col(lam)
    y = np.linalg.det(F) - 1.0
    c = cofactor(F).reshape(t, d * d)
    return (2.0 * arap_hessian_element_F(F, mu)
            + lam[:, None, None] * c[:, :, None] * c[:, None, :]
            + (lam * y)[:, None, None] * det_hessian(F))


class _Assembled:
    """energy_x / gradient_x / hessian_x with the (x, J, mu, lam, vol) signature the
    rollout uses; ARAP ignores lam."""

    def __init__(self, psi, pk1, hess):
        self._psi, self._pk1, self._hess = psi, pk1, hess

    def energy_x(self, x, J, mu, lam, vol) -> float:
        F = _F_of(x, J, _dim_of(J, x))
        return float((np.asarray(vol).reshape(-1, 1) * self._psi(F, mu, lam)).sum())

    def gradient_x(self, x, J, mu, lam, vol) -> np.ndarray:
        F = _F_of(x, J, _dim_of(J, x))
        P = self._pk1(F, mu, lam) * np.asarray(vol).reshape(-1, 1, 1)
        return J.T @ P.reshape(-1, 1)

    def hessian_x(self, x, J, mu, lam, vol, psd: bool = True):
        F = _F_of(x, J, _dim_of(J, x))
        He = self._hess(F, mu, lam) * np.asarray(vol).reshape(-1, 1, 1)
        if psd:
            He = psd_project(He)
        return (J.T @ _block_diag(He) @ J).tocsr()


arap = _Assembled(lambda F, mu, lam: arap_energy_element_F(F, mu),
                  lambda F, mu, lam: arap_gradient_element_F(F, mu),
                  lambda F, mu, lam: arap_hessian_element_F(F, mu))
fcr = _Assembled(fcr_energy_element_F, fcr_gradient_element_F, fcr_hessian_element_F)
