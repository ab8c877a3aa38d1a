"""Macklin-Mueller neo-Hookean element and assembled tiers, FP64 restatement.

Test infrastructure only: the checker of the GPU kernels, never the measured or
shipped path.

Energy density (Macklin and Mueller 2021), as simkit writes it in
``simkit/energies/macklin_mueller_neo_hookean.py:66-122``::

    psi(F) = mu (1 - J) + lam/2 (1 - J)^2 + mu/2 (I_C - d)
    P(F)   = mu F + D cof(F),         D = lam (J - 1) - mu     (:125-185)
    H(F)   = mu I + lam c c^T + D d2J/dF2                        (:188-374)

with ``c = vec(cof F)`` row-major.  simkit expands these entrywise from
generated code; here they follow from dpsi/dI_C = mu/2 and dpsi/dJ = D, with the
determinant's derivatives from ``oracle.snh``.  The assembled tiers weight by
``vol``, optionally PSD-project the weighted blocks and assemble
``J^T blockdiag(He) J`` (:484-574), the same composition as the stable
neo-Hookean path.
"""

from __future__ import annotations

import numpy as np

from .psd import psd_project
from .snh import _F_of, _block_diag, _dim_of, _invariants, cofactor, det_hessian


def _mat(F, mu, lam):
    F = np.asarray(F, dtype=np.float64)
    d = F.shape[-1]
    if d not in (2, 3):
        raise ValueError("Macklin-Mueller Neo-Hookean supports dim=2 or dim=3")
    F = F.reshape(-1, d, d)
    mu = np.asarray(mu, dtype=np.float64).reshape(-1)
    lam = np.asarray(lam, dtype=np.float64).reshape(-1)
    return F, d, mu, lam


def energy_element_F(F, mu, lam) -> np.ndarray:
    """psi per element, (t, 1).  Reference: ``macklin_mueller_neo_hookean.py:66-122``."""
    F, d, mu, lam = _mat(F, mu, lam)
    IC, J = _invariants(F)
    e = 1.0 - J
    return (mu * e + 0.5 * lam * e * e + 0.5 * mu * (IC - d)).reshape(-1, 1)


def gradient_element_F(F, mu, lam) -> np.ndarray:
    """PK1 per element, (t, d, d).  Reference: ``:125-185``."""
    F, d, mu, lam = _mat(F, mu, lam)
    _, J = _invariants(F)
    D = lam * (J - 1.0) - mu
    return mu[:, None, None] * F + D[:, None, None] * cofactor(F)


def hessian_element_F(F, mu, lam) -> np.ndarray:
    """d*d x d*d F-Hessian per element, not projected.  Reference: ``:188-374``."""
    F, d, mu, lam = _mat(F, mu, lam)
    t = F.shape[0]
    _, J = _invariants(F)
    D = lam * (J - 1.0) - mu
    c = cofactor(F).reshape(t, d * d)
    return (mu[:, None, None] * np.eye(d * d)[None]
            + lam[:, None, None] * c[:, :, None] * c[:, None, :]
            + D[:, None, None] * det_hessian(F))


def energy_x(x, J, mu, lam, vol) -> float:
    """sum_e vol_e psi(F_e), F = J x.  Reference: ``:484-509``."""
    F = _F_of(x, J, _dim_of(J, x))
    return float((np.asarray(vol).reshape(-1, 1) * energy_element_F(F, mu, lam)).sum())


def gradient_x(x, J, mu, lam, vol) -> np.ndarray:
    """J^T vec(vol P).  Reference: ``:512-538``."""
    F = _F_of(x, J, _dim_of(J, x))
    P = gradient_element_F(F, mu, lam) * np.asarray(vol).reshape(-1, 1, 1)
    return J.T @ P.reshape(-1, 1)


def hessian_x(x, J, mu, lam, vol, psd: bool = True):
    """J^T blockdiag(psd(vol He)) J.  Reference: ``:541-574``."""
    F = _F_of(x, J, _dim_of(J, x))
    He = hessian_element_F(F, mu, lam) * np.asarray(vol).reshape(-1, 1, 1)
    if psd:
        He = psd_project(He)
    return (J.T @ _block_diag(He) @ J).tocsr()
