"""Armijo backtracking, Newton and backward Euler, FP64 restatement.

These follow simkit's control flow statement by statement, so the oracle
takes the same steps the reference takes on the same inputs.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sps
import scipy.sparse.linalg as spla
import scipy.linalg as sla


def backtracking_line_search(f, x0, g, dx, alpha=0.01, beta=0.5, max_iter=100, threshold=1e-12):
    """Reference: ``simkit/backtracking_line_search.py:8-67``.

    t starts at 1 and is multiplied by ``beta`` until
    ``f(x0 + t dx) <= f(x0) + alpha t g^T dx + threshold``; after ``max_iter``
    failures the result is ``(0, x0, f(x0))``.
    """
    assert 0 < alpha <= 0.5
    assert 0 < beta < 1
    assert np.ndim(x0) == np.ndim(dx)
    fx0 = f(x0)
    slope = g.T @ dx
    t = 1.0
    for _ in range(max_iter):
        x = x0 + t * dx
        fx = f(x)
        if fx <= fx0 + alpha * t * slope + threshold:
            return t, x, fx
        t *= beta
    return 0.0, x0, fx0


def newton_solver(x0, energy_func, gradient_func, hessian_func, tolerance=1e-6,
                  max_iter=1, do_line_search=True, return_info=False):
    """Reference: ``simkit/solvers/newton.py:7-75``.  Direct sparse solve (SuperLU)."""
    x = x0.copy()
    info = {"g": [], "dx": [], "alphas": [], "iters": -1}
    for i in range(max_iter):
        g = gradient_func(x)
        H = hessian_func(x)
        if sps.issparse(H):
            dx = spla.spsolve(H.tocsc(), -g).reshape(-1, 1)
        else:
            dx = sla.solve(H, -g).reshape(-1, 1)
        alpha = backtracking_line_search(energy_func, x, g, dx)[0] if do_line_search else 1.0
        x += alpha * dx
        info["g"].append(g)
        info["dx"].append(dx)
        info["alphas"].append(alpha)
        info["iters"] = i
        if np.linalg.norm(alpha * dx) < tolerance:
            break
    return (x, info) if return_info else x


# kinetic term of backward Euler: simkit/energies/kinetic.py:87-194
def be_target(x_curr, x_prev, h):
    """x_curr + h (x_curr - x_prev)/h.  Reference: ``kinetic.py:87-90``."""
    return x_curr + h * ((x_curr - x_prev) / h)


def kinetic_energy_be(x, x_curr, x_prev, M, h):
    d = x - be_target(x_curr, x_prev, h)
    return float((0.5 * (d.T @ (M @ d)) / h ** 2).item())


def kinetic_gradient_be(x, x_curr, x_prev, M, h):
    return (M @ (x - be_target(x_curr, x_prev, h))) / h ** 2


def kinetic_hessian_be(M, h):
    return M / h ** 2


def backward_euler(x_curr, x_prev, energy_func, gradient_func, hessian_func, M, h,
                   tolerance=1e-6, max_iter=1, do_line_search=True, return_info=False):
    """Reference: ``simkit/integrators/backward_euler.py:27-91``."""
    def energy(x):
        return energy_func(x) + kinetic_energy_be(x, x_curr, x_prev, M, h)

    def gradient(x):
        return gradient_func(x) + kinetic_gradient_be(x, x_curr, x_prev, M, h)

    def hessian(x):
        return hessian_func(x) + kinetic_hessian_be(M, h)

    x0 = be_target(x_curr, x_prev, h)
    return newton_solver(x0, energy, gradient, hessian, tolerance=tolerance, max_iter=max_iter,
                         do_line_search=do_line_search, return_info=return_info)


# BDF2: simkit/integrators/bdf2.py:31-101, simkit/energies/kinetic.py:63-101, 200-279
BDF2_COEFF = 9.0 / 4.0   # kinetic.py:35


def velocity_bdf2(x_curr, x_prev, x_prev2, h):
    """(3 x_curr - 4 x_prev + x_prev2) / (2h).  Reference: ``kinetic.py:63-84``."""
    return (3.0 * x_curr - 4.0 * x_prev + x_prev2) / (2.0 * h)


def bdf2_target(x_curr, x_prev, x_prev2, x_prev3, h):
    """(4/3) x_curr - (1/3) x_prev + (8h/9) v_curr - (2h/9) v_prev.  Reference: ``kinetic.py:93-101``."""
    v_curr = velocity_bdf2(x_curr, x_prev, x_prev2, h)
    v_prev = velocity_bdf2(x_prev, x_prev2, x_prev3, h)
    return (4.0 / 3.0) * x_curr - (1.0 / 3.0) * x_prev + (8.0 * h / 9.0) * v_curr - (2.0 * h / 9.0) * v_prev


def kinetic_energy_bdf2(x, x_curr, x_prev, x_prev2, x_prev3, M, h):
    d = x - bdf2_target(x_curr, x_prev, x_prev2, x_prev3, h)
    return float((0.5 * BDF2_COEFF * (d.T @ (M @ d)) / h ** 2).item())


def kinetic_gradient_bdf2(x, x_curr, x_prev, x_prev2, x_prev3, M, h):
    return BDF2_COEFF * (M @ (x - bdf2_target(x_curr, x_prev, x_prev2, x_prev3, h))) / h ** 2


def kinetic_hessian_bdf2(M, h):
    return BDF2_COEFF * M / h ** 2


def bdf2(x_curr, x_prev, x_prev2, x_prev3, energy_func, gradient_func, hessian_func, M, h,
         tolerance=1e-6, max_iter=1, do_line_search=True, return_info=False):
    """Reference: ``simkit/integrators/bdf2.py:31-101``."""
    def energy(x):
        return energy_func(x) + kinetic_energy_bdf2(x, x_curr, x_prev, x_prev2, x_prev3, M, h)

    def gradient(x):
        return gradient_func(x) + kinetic_gradient_bdf2(x, x_curr, x_prev, x_prev2, x_prev3, M, h)

    def hessian(x):
        return hessian_func(x) + kinetic_hessian_bdf2(M, h)

    x0 = bdf2_target(x_curr, x_prev, x_prev2, x_prev3, h)
    return newton_solver(x0, energy, gradient, hessian, tolerance=tolerance, max_iter=max_iter,
                         do_line_search=do_line_search, return_info=return_info)
