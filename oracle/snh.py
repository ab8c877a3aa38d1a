"""Stable neo-Hookean element and assembled tiers, FP64 restatement.

Energy density (Smith, de Goes, Kim 2018), as simkit writes it in
``simkit/energies/stable_neo_hookean.py:65-129``::

    psi(F)  = mu/2 (I_C - d) - mu/2 log(I_C + 1) + lam/2 (J - alpha)^2
    alpha   = 1 + d mu / ((d + 1) lam)                   (:88)
    P(F)    = A F + D cof(F),  A = mu I_C/(I_C+1),  D = lam (J - alpha)   (:192-215)
    H(F)    = A I + B f f^T + lam c c^T + D d2J/dF2,  B = 2 mu/(I_C+1)^2  (:315-440)

with ``f = vec(F)`` and ``c = vec(cof F)`` in row-major order (the order simkit
produces after its ``mat2py`` permutation, ``simkit/mat2py.py:19-31``).  The
second derivative of the determinant is written with Levi-Civita symbols
instead of simkit's 81 hand-expanded entries; the values are the same up to
FP64 rounding.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sps

from .psd import psd_project


def _levi_civita3() -> np.ndarray:
    e = np.zeros((3, 3, 3))
    e[0, 1, 2] = e[1, 2, 0] = e[2, 0, 1] = 1.0
    e[0, 2, 1] = e[2, 1, 0] = e[1, 0, 2] = -1.0
    return e


_EPS3 = _levi_civita3()
_EPS2 = np.array([[0.0, 1.0], [-1.0, 0.0]])


def _invariants(F: np.ndarray):
    d = F.shape[-1]
    if d not in (2, 3):
        raise ValueError("Stable Neo-Hookean supports dim=2 or dim=3")
    IC = np.einsum("tij,tij->t", F, F)
    if d == 2:
        J = F[:, 0, 0] * F[:, 1, 1] - F[:, 0, 1] * F[:, 1, 0]
    else:
        J = (F[:, 0, 0] * (F[:, 1, 1] * F[:, 2, 2] - F[:, 1, 2] * F[:, 2, 1])
             - F[:, 0, 1] * (F[:, 1, 0] * F[:, 2, 2] - F[:, 1, 2] * F[:, 2, 0])
             + F[:, 0, 2] * (F[:, 1, 0] * F[:, 2, 1] - F[:, 1, 1] * F[:, 2, 0]))
    return IC, J


def cofactor(F: np.ndarray) -> np.ndarray:
    """cof(F) = dJ/dF, row-major, per element (simkit ``snh.py:200-208``)."""
    d = F.shape[-1]
    if d == 2:
        C = np.empty_like(F)
        C[:, 0, 0] = F[:, 1, 1]
        C[:, 0, 1] = -F[:, 1, 0]
        C[:, 1, 0] = -F[:, 0, 1]
        C[:, 1, 1] = F[:, 0, 0]
        return C
    # cof_ij = 1/2 eps_imn eps_jpq F_mp F_nq
    return 0.5 * np.einsum("imn,jpq,tmp,tnq->tij", _EPS3, _EPS3, F, F)


def _params(F, mu, lam):
    d = F.shape[-1]
    mu = np.asarray(mu, dtype=np.float64).reshape(-1)
    lam = np.asarray(lam, dtype=np.float64).reshape(-1)
    alpha = 1.0 + d * mu / ((d + 1) * lam)
    return d, mu, lam, alpha


def energy_element_F(F, mu, lam) -> np.ndarray:
    """psi per element, shape (t, 1).  Reference: ``snh.py:65-129``."""
    F = np.asarray(F, dtype=np.float64)
    d = F.shape[-1]
    F = F.reshape(-1, d, d)
    d, mu, lam, alpha = _params(F, mu, lam)
    IC, J = _invariants(F)
    psi = 0.5 * mu * (IC - d) - 0.5 * mu * np.log(IC + 1.0) + 0.5 * lam * (J - alpha) ** 2
    return psi.reshape(-1, 1)


def gradient_element_F(F, mu, lam) -> np.ndarray:
    """PK1 per element, shape (t, d, d).  Reference: ``snh.py:132-218``."""
    F = np.asarray(F, dtype=np.float64)
    d = F.shape[-1]
    F = F.reshape(-1, d, d)
    d, mu, lam, alpha = _params(F, mu, lam)
    IC, J = _invariants(F)
    A = mu * IC / (IC + 1.0)
    D = lam * (J - alpha)
    return A[:, None, None] * F + D[:, None, None] * cofactor(F)


def det_hessian(F: np.ndarray) -> np.ndarray:
    """d^2 det(F) / dF^2 in row-major vec(F) order, shape (t, d*d, d*d)."""
    d = F.shape[-1]
    t = F.shape[0]
    if d == 2:
        HJ = np.einsum("ik,jl->ijkl", _EPS2, _EPS2)
        return np.broadcast_to(HJ.reshape(1, 4, 4), (t, 4, 4)).copy()
    HJ = np.einsum("ikm,jln,tmn->tijkl", _EPS3, _EPS3, F)
    return HJ.reshape(t, 9, 9)


def hessian_element_F(F, mu, lam) -> np.ndarray:
    """9x9 (or 4x4) F-Hessian per element, not projected.  Reference: ``snh.py:221-443``."""
    F = np.asarray(F, dtype=np.float64)
    d = F.shape[-1]
    F = F.reshape(-1, d, d)
    d, mu, lam, alpha = _params(F, mu, lam)
    t = F.shape[0]
    IC, J = _invariants(F)
    A = mu * IC / (IC + 1.0)
    B = 2.0 * mu / (IC + 1.0) ** 2
    D = lam * (J - alpha)
    f = F.reshape(t, d * d)
    c = cofactor(F).reshape(t, d * d)
    H = (A[:, None, None] * np.eye(d * d)[None]
         + B[:, None, None] * f[:, :, None] * f[:, None, :]
         + lam[:, None, None] * c[:, :, None] * c[:, None, :]
         + D[:, None, None] * det_hessian(F))
    return H


# --------------------------------------------------------------------------- #
# assembled tier (x variable); reference ``snh.py:449-538``                    #
# --------------------------------------------------------------------------- #
def _F_of(x, J, d):
    return (J @ np.asarray(x, dtype=np.float64).reshape(-1, 1)).reshape(-1, d, d)


def energy_x(x, J, mu, lam, vol) -> float:
    """sum_e vol_e psi(F_e) with F = J x.  Reference: ``snh.py:449-474``."""
    d = _dim_of(J, x)
    F = _F_of(x, J, d)
    return float((np.asarray(vol).reshape(-1, 1) * energy_element_F(F, mu, lam)).sum())


def gradient_x(x, J, mu, lam, vol) -> np.ndarray:
    """J^T vec(vol P).  Reference: ``snh.py:477-503``."""
    d = _dim_of(J, x)
    F = _F_of(x, J, d)
    P = gradient_element_F(F, mu, lam) * np.asarray(vol).reshape(-1, 1, 1)
    return J.T @ P.reshape(-1, 1)


def hessian_x(x, J, mu, lam, vol, psd: bool = True):
    """J^T blockdiag(psd(vol He)) J.  Reference: ``snh.py:506-538``."""
    d = _dim_of(J, x)
    F = _F_of(x, J, d)
    He = hessian_element_F(F, mu, lam) * np.asarray(vol).reshape(-1, 1, 1)
    if psd:
        He = psd_project(He)
    return (J.T @ _block_diag(He) @ J).tocsr()


def _block_diag(He):
    """scipy block_diag of a (t, k, k) stack, as snh.py:536 builds it."""
    t, k, _ = He.shape
    r = (np.arange(t)[:, None, None] * k + np.arange(k)[None, :, None]).repeat(k, axis=2)
    c = (np.arange(t)[:, None, None] * k + np.arange(k)[None, None, :]).repeat(k, axis=1)
    return sps.csr_matrix((He.ravel(), (r.ravel(), c.ravel())), shape=(t * k, t * k))


def element_hessians_projected(x, J, mu, lam, vol) -> np.ndarray:
    """The vol-weighted, PSD-projected F-space blocks that ``hessian_x`` assembles."""
    d = _dim_of(J, x)
    F = _F_of(x, J, d)
    He = hessian_element_F(F, mu, lam) * np.asarray(vol).reshape(-1, 1, 1)
    return psd_project(He)


def _dim_of(J, x) -> int:
    """Spatial dimension: from ``x`` of shape (n, d) as the reference takes it,
    else 3 for flattened (d n, 1) positions (the backward-Euler closures)."""
    x = np.asarray(x)
    if x.ndim == 2 and x.shape[1] in (2, 3) and x.shape[0] * x.shape[1] == J.shape[1]:
        return x.shape[1]
    return 3
