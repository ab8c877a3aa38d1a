"""The displacement (_u) tier of every energy, FP64 restatement.

Test infrastructure only: the checker of the GPU kernels, never the measured or
shipped path.

simkit's ``*_energy_u`` / ``*_gradient_u`` / ``*_hessian_u`` (stable_neo_hookean.py:544-648,
macklin_mueller_neo_hookean.py:579-683, arap.py:331-424, fcr.py:403-502, dispatched by
elastic.py:151-746) evaluate the ``_x`` tier at F = J u + Jx_bar, where Jx_bar = J x_bar is a
precomputed deformation gradient of an arbitrary reference pose; dF/du = J, so the gradient is
J^T vec(vol P) and the Hessian J^T blockdiag(psd(vol He)) J as in the ``_x`` tier.
"""

from __future__ import annotations

import numpy as np

from . import corot, linel, mmnh, snh
from .psd import psd_project
from .snh import _block_diag

# element functions (F, mu, lam) of each material
ELEMENT = {
    "snh": (snh.energy_element_F, snh.gradient_element_F, snh.hessian_element_F),
    "mmnh": (mmnh.energy_element_F, mmnh.gradient_element_F, mmnh.hessian_element_F),
    "arap": (corot.arap._psi, corot.arap._pk1, corot.arap._hess),
    "fcr": (corot.fcr._psi, corot.fcr._pk1, corot.fcr._hess),
    "le": (linel.energy_element_F, linel.gradient_element_F, linel.hessian_element_F),
}
NEVER_PROJECTED = {"le"}   # linear_elasticity_hessian_u ignores psd (linear_elasticity.py:301-333)


def _F(u, J, Jx_bar):
    u = np.asarray(u, dtype=np.float64)
    d = u.shape[1] if u.ndim == 2 else 3
    return (J @ u.reshape(-1, 1) + np.asarray(Jx_bar, dtype=np.float64).reshape(-1, 1)).reshape(-1, d, d)


def energy_u(material, u, J, Jx_bar, mu, lam, vol) -> float:
    F = _F(u, J, Jx_bar)
    return float((np.asarray(vol).reshape(-1, 1) * ELEMENT[material][0](F, mu, lam)).sum())


def gradient_u(material, u, J, Jx_bar, mu, lam, vol) -> np.ndarray:
    F = _F(u, J, Jx_bar)
    P = ELEMENT[material][1](F, mu, lam) * np.asarray(vol).reshape(-1, 1, 1)
    return J.T @ P.reshape(-1, 1)


def hessian_u(material, u, J, Jx_bar, mu, lam, vol, psd: bool = True):
    F = _F(u, J, Jx_bar)
    He = ELEMENT[material][2](F, mu, lam) * np.asarray(vol).reshape(-1, 1, 1)
    if psd and material not in NEVER_PROJECTED:
        He = psd_project(He)
    return (J.T @ _block_diag(He) @ J).tocsr()
