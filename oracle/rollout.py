"""Backward-Euler (or BDF2) rollout of a pinned beam, as simkit would run it.

The step is simkit's own composition (``simkit/integrators/backward_euler.py:76-91``
around ``simkit/solvers/newton.py:46-69``): energy, gradient and Hessian
closures are the stable neo-Hookean ``_x`` tier plus the gravity potential
``-f^T x`` plus the backward-Euler kinetic term, and each Newton iteration is
``spsolve`` + Armijo backtracking.  Two harness rules make the stopping point
well defined:

1. Free-DOF elimination.  Pinned DOFs stay at rest and Newton runs on the
   free DOFs (Hessian ``S K S^T`` for the free selector ``S``).  This is the
   limit of simkit's penalty pin (``simkit/dirichlet_penalty.py:115-142``)
   without its large cancelling constant.
2. Relative-residual stop.  ``newton_solver(..., max_iter=1)`` is called
   repeatedly (each call is one reference Newton iteration) until
   ``||g_free(y)|| / ||g_free(y_tilde)|| < tol`` or ``max_newton`` calls.

BDF2 (``simkit/integrators/bdf2.py:31-101``) differs only in the inertial
target (``kinetic.py:93-101``, from four position levels) and the factor
c = 9/4 on the kinetic term; from rest every history level is the rest shape.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.sparse as sps

from . import contact, corot, fem, linel, mmnh, snh
from .solvers import BDF2_COEFF, bdf2_target, newton_solver, be_target


@dataclass
class StepInfo:
    iters: int
    residuals: list
    alphas: list
    converged: bool


class BeamRollout:
    """FP64 reference rollout of one beam instance."""

    def __init__(self, X, T, mu, lam, rho, gravity, pinned, dt, tol=1e-6, max_newton=20, material="snh",
                 planes=None, contact_mass_weighted=True):
        # the elastic energy: 'snh' (stable_neo_hookean.py), 'mmnh' (macklin_mueller_neo_hookean.py),
        # 'arap' (arap.py), 'fcr' (fcr.py) or 'le' (linear_elasticity.py)
        self.energy = {"snh": snh, "mmnh": mmnh, "arap": corot.arap, "fcr": corot.fcr, "le": linel}[material]
        # contact springs (contact_springs_plane.py): (k, p, n) per plane, weights = vertex masses or 1
        self.planes = list(planes or [])
        self.contact_mass_weighted = contact_mass_weighted
        self.X = np.asarray(X, dtype=np.float64)
        self.T = np.asarray(T)
        self.mu = np.asarray(mu, dtype=np.float64).reshape(-1, 1)
        self.lam = np.asarray(lam, dtype=np.float64).reshape(-1, 1)
        self.dt = float(dt)
        self.tol = float(tol)
        self.max_newton = int(max_newton)
        n = self.X.shape[0]
        self.n = n
        self.J = fem.deformation_jacobian(self.X, self.T)
        self.vol = fem.tet_volumes(self.X, self.T)
        m = fem.lumped_mass(self.X, self.T, rho)
        self.mass = m
        self.f_ext = (m[:, None] * np.asarray(gravity, dtype=np.float64)[None, :]).reshape(-1, 1)
        pinned_v = np.asarray(pinned).ravel()
        pin_dofs = (3 * pinned_v[:, None] + np.arange(3)[None, :]).ravel()
        mask = np.ones(3 * n, dtype=bool)
        mask[pin_dofs] = False
        self.free = np.nonzero(mask)[0]
        self.S = fem.selection_matrix(self.free, 3 * n)          # free selector
        self.M = sps.diags(np.repeat(m, 3)).tocsc()
        self.Mf = (self.S @ self.M @ self.S.T).tocsc()
        self.x_rest = self.X.reshape(-1, 1).copy()

    # full positions from free DOFs (pinned DOFs at rest)
    def full(self, y):
        x = self.x_rest.copy()
        x[self.free] = y
        return x

    def _contact_M(self):
        return sps.diags(self.mass) if self.contact_mass_weighted else None

    def contact_energy(self, x):
        return sum(contact.energy(x, k, p, n, self._contact_M()) for k, p, n in self.planes)

    def contact_gradient(self, x):
        return sum(contact.gradient(x, k, p, n, self._contact_M()) for k, p, n in self.planes)

    def contact_hessian(self, x):
        return sum(contact.hessian(x, k, p, n, self._contact_M()) for k, p, n in self.planes)

    def potential(self, x) -> float:
        e = self.energy.energy_x(x, self.J, self.mu, self.lam, self.vol) - (self.f_ext.T @ x).item()
        return e + (self.contact_energy(x) if self.planes else 0.0)

    def potential_gradient(self, x):
        g = self.energy.gradient_x(x, self.J, self.mu, self.lam, self.vol) - self.f_ext
        return g + self.contact_gradient(x) if self.planes else g

    def potential_hessian(self, x):
        K = self.energy.hessian_x(x, self.J, self.mu, self.lam, self.vol)
        return (K + self.contact_hessian(x)).tocsr() if self.planes else K

    # inertial targets (overridable to plug in another implementation of the same formulas)
    def be_target(self, yc, yp, h):
        return be_target(yc, yp, h)

    def bdf2_target(self, yc, yp, yp2, yp3, h):
        return bdf2_target(yc, yp, yp2, yp3, h)

    def step(self, x_curr, x_prev, newton=newton_solver, x_prev2=None, x_prev3=None):
        """One backward-Euler step, or a BDF2 step when x_prev2 and x_prev3 are given;
        returns (x_next (3n,1), StepInfo)."""
        h = self.dt
        yc = x_curr[self.free]
        yp = x_prev[self.free]
        if x_prev2 is None:
            y_tilde = self.be_target(yc, yp, h)
            c = 1.0
        else:
            y_tilde = self.bdf2_target(yc, yp, x_prev2[self.free], x_prev3[self.free], h)
            c = BDF2_COEFF
        Mf = self.Mf

        def E(y):
            d = y - y_tilde
            return self.potential(self.full(y)) + float((0.5 * c * (d.T @ (Mf @ d)) / h ** 2).item())

        def G(y):
            return self.S @ self.potential_gradient(self.full(y)) + c * (Mf @ (y - y_tilde)) / h ** 2

        def H(y):
            K = self.potential_hessian(self.full(y))
            return (self.S @ K @ self.S.T + c * Mf / h ** 2).tocsc()

        y = y_tilde.copy()
        g0 = float(np.linalg.norm(G(y)))
        res = [1.0 if g0 > 0 else 0.0]
        alphas = []
        it = 0
        while res[-1] >= self.tol and it < self.max_newton and g0 > 0:
            y, info = newton(y, E, G, H, max_iter=1, return_info=True)
            alphas.append(info["alphas"][0])
            it += 1
            res.append(float(np.linalg.norm(G(y))) / g0)
        return self.full(y), StepInfo(iters=it, residuals=res, alphas=alphas,
                                      converged=res[-1] < self.tol)

    def elastic_energy(self, x) -> float:
        return self.energy.energy_x(x, self.J, self.mu, self.lam, self.vol)

    def rollout(self, steps, record=None, integrator="be"):
        """Run ``steps`` steps from rest ('be' or 'bdf2'); returns positions (steps+1, 3n) and
        per-step infos."""
        x_prev3 = self.x_rest.copy()
        x_prev2 = self.x_rest.copy()
        x_prev = self.x_rest.copy()
        x_curr = self.x_rest.copy()
        xs = [x_curr.ravel().copy()]
        infos = []
        for s in range(steps):
            if integrator == "bdf2":
                x_next, info = self.step(x_curr, x_prev, x_prev2=x_prev2, x_prev3=x_prev3)
            else:
                x_next, info = self.step(x_curr, x_prev)
            infos.append(info)
            xs.append(x_next.ravel().copy())
            x_prev3, x_prev2, x_prev, x_curr = x_prev2, x_prev, x_curr, x_next
            if record is not None:
                record(s, x_next, info)
        return np.array(xs), infos


def from_spec(spec, dt=1.0 / 60.0, tol=1e-6, max_newton=20, material="snh", planes=None,
              contact_mass_weighted=True) -> BeamRollout:
    return BeamRollout(spec.X, spec.T, spec.mu, spec.lam, spec.rho, spec.gravity, spec.pinned,
                       dt, tol=tol, max_newton=max_newton, material=material, planes=planes,
                       contact_mass_weighted=contact_mass_weighted)
