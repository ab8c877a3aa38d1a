"""Generate the golden fixtures of the FEM path by running simkit itself.

Usage::

    SIMKIT_REFERENCE=/path/to/simkit/checkout python tests/golden/make_golden.py [--skip-c1] [--skip-c2]
    python tests/golden/make_golden.py --reference /path/to/simkit/checkout --only c2

Every number stored here comes out of the reference's own functions
(``simkit.energies.stable_neo_hookean``, ``simkit.psd_project``,
``simkit.deformation_jacobian``, ``simkit.volume``, ``simkit.massmatrix``,
``simkit.solvers.newton_solver``); inputs are seeded.  The rollout fixtures use
the harness rules of ``oracle/rollout.py`` (free-DOF elimination, relative
residual stop) with the reference's math plugged in.

Fixtures written next to this script:

* ``element_3d.npz`` / ``element_2d.npz``: F, mu, lam, vol -> psi, P, He, psd(vol He)
* ``beam_small.npz``: 4x2x2 jittered beam: J (csc), vol, mass, energy/gradient/Hessian at a perturbed x
* ``rollout_small.npz``: 6x2x2 beam, 8 backward-Euler steps (positions, iterations, residuals)
* ``rollout_beam_8x8x32.npz``: the 12,288-tet beam, 60 steps (displacements at a few steps, energies, iterations)
* ``rollout_bdf2_small.npz``: 6x2x2 beam, 8 BDF2 steps from rest (the reference's BDF2 target and coefficient)
* ``element_mmnh_3d.npz`` / ``element_mmnh_2d.npz``: Macklin-Mueller neo-Hookean element tier on the same F batches
* ``rollout_mmnh_small.npz``: 6x2x2 beam, 8 backward-Euler steps with the Macklin-Mueller energy
* ``element_arap_{3d,2d}.npz`` / ``element_fcr_{3d,2d}.npz``: ARAP and fixed-corotated element tiers on the same F batches
* ``rollout_arap_small.npz`` / ``rollout_fcr_small.npz``: 6x2x2 beam, 8 backward-Euler steps with those energies
* ``element_le_{3d,2d}.npz`` / ``rollout_le_small.npz``: the same for linear elasticity
* ``beam_u_tier.npz``: 3x2x2 jittered beam: the displacement (_u) tier of all four energies (F = J u + J x_bar
  with x_bar a perturbed pose): energies, gradients and projected / unprojected Hessians
* ``contact_plane.npz``: contact springs energy / gradient / Hessian of seeded points against a plane
* ``rollout_contact_small.npz``: 6x2x2 beam falling onto a floor plane (contact springs), 14 steps
* ``cache_reference.npz``: a cache file written by simkit's compute_with_cache_check (array, scalar, 1-element array)
* ``rollout_beam_32x32x128_first_steps.npz``: the 786,432-tet jittered beam with E log-uniform [1e5, 1e7], the first
  two steps from rest (sampled vertices), with simkit's spsolve replaced by a 1e-10 PCG (labelled in the file)
"""

from __future__ import annotations

import argparse
import os
import sys
import time
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)


def _import_reference(path):
    sys.path.insert(0, path)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        import simkit  # noqa: F401
        from simkit.energies import stable_neo_hookean as ref_snh
        from simkit.psd_project import psd_project
        from simkit.deformation_jacobian import deformation_jacobian
        from simkit.volume import volume
        from simkit.massmatrix import massmatrix
        from simkit.solvers import newton_solver
        from simkit.energies import kinetic
        from simkit.energies import macklin_mueller_neo_hookean as ref_mmnh
        from simkit.energies import contact_springs_plane as ref_contact
        from simkit.energies import arap as ref_arap
        from simkit.energies import fcr as ref_fcr
        from simkit.energies import linear_elasticity as ref_le
    return dict(le=ref_le, snh=ref_snh, psd_project=psd_project, deformation_jacobian=deformation_jacobian,
                volume=volume, massmatrix=massmatrix, newton_solver=newton_solver, kinetic=kinetic,
                mmnh=ref_mmnh, contact=ref_contact, arap=ref_arap, fcr=ref_fcr)


def element_cases(rng, d, t_each=32):
    """Seeded F batches spanning rest, small/large strain, inversion and collapse."""
    eye = np.eye(d)[None]
    cases = [
        np.repeat(eye, 4, axis=0),                                   # exact rest
        eye + 0.05 * rng.standard_normal((t_each, d, d)),           # the reference test's scale
        eye + 0.3 * rng.standard_normal((t_each, d, d)),
        eye + 1.0 * rng.standard_normal((t_each, d, d)),
    ]
    inv = eye + 0.2 * rng.standard_normal((t_each, d, d))
    inv[:, :, 0] *= -1.0                                             # inverted (J < 0)
    cases.append(inv)
    col = eye + 0.05 * rng.standard_normal((t_each, d, d))
    col[:, :, -1] *= 0.05                                           # nearly collapsed (J ~ 0.05)
    cases.append(col)
    # random rotations times small stretch
    q, _ = np.linalg.qr(rng.standard_normal((t_each, d, d)))
    q *= np.sign(np.linalg.det(q))[:, None, None]
    cases.append(q @ (eye + 0.02 * rng.standard_normal((t_each, d, d))))
    F = np.concatenate(cases, axis=0)
    t = F.shape[0]
    ym = np.exp(rng.uniform(np.log(1e5), np.log(1e7), size=(t, 1)))
    pr = rng.uniform(0.30, 0.49, size=(t, 1))
    mu = ym / (2 * (1 + pr))
    lam = ym * pr / ((1 + pr) * (1 - 2 * pr))
    vol = rng.uniform(1e-7, 5e-6, size=(t, 1))
    return F, mu, lam, vol


def make_element(ref, d, out):
    rng = np.random.default_rng(100 + d)
    F, mu, lam, vol = element_cases(rng, d)
    s = ref["snh"]
    psi = s.stable_neo_hookean_energy_element_F(F, mu, lam)
    P = s.stable_neo_hookean_gradient_element_F(F, mu, lam)
    He = s.stable_neo_hookean_hessian_element_F(F, mu, lam)
    Hp = ref["psd_project"](He * vol.reshape(-1, 1, 1))
    np.savez_compressed(out, F=F, mu=mu, lam=lam, vol=vol, psi=psi, P=P, He=He, He_proj=Hp)


def make_element_mmnh(ref, d, out):
    rng = np.random.default_rng(100 + d)
    F, mu, lam, vol = element_cases(rng, d)
    m = ref["mmnh"]
    psi = m.macklin_mueller_neo_hookean_energy_element_F(F, mu, lam)
    P = m.macklin_mueller_neo_hookean_gradient_element_F(F, mu, lam)
    He = m.macklin_mueller_neo_hookean_hessian_element_F(F, mu, lam)
    Hp = ref["psd_project"](He * vol.reshape(-1, 1, 1))
    np.savez_compressed(out, F=F, mu=mu, lam=lam, vol=vol, psi=psi, P=P, He=He, He_proj=Hp)


def make_element_corot(ref, d, out, material):
    """ARAP (lam stored but unused) or fixed-corotated element tier."""
    rng = np.random.default_rng(100 + d)
    F, mu, lam, vol = element_cases(rng, d)
    if material == "arap":
        a = ref["arap"]
        psi = a.arap_energy_element_F(F, mu)
        P = a.arap_gradient_element_F(F, mu)
        He = a.arap_hessian_element_F(F, mu)
    else:
        f = ref["fcr"]
        psi = f.fcr_energy_element_F(F, mu, lam)
        P = f.fcr_gradient_element_F(F, mu, lam)
        He = f.fcr_hessian_element_F(F, mu, lam)
    Hp = ref["psd_project"](He * vol.reshape(-1, 1, 1))
    np.savez_compressed(out, F=F, mu=mu, lam=lam, vol=vol, psi=psi, P=P, He=He, He_proj=Hp)


def make_element_le(ref, d, out):
    rng = np.random.default_rng(100 + d)
    F, mu, lam, vol = element_cases(rng, d)
    m = ref["le"]
    psi = m.linear_elasticity_energy_element_F(F, mu, lam)
    P = m.linear_elasticity_gradient_element_F(F, mu, lam)
    He = m.linear_elasticity_hessian_element_F(F, mu, lam)
    np.savez_compressed(out, F=F, mu=mu, lam=lam, vol=vol, psi=psi, P=P, He=He)


def make_beam_small(ref, out):
    from simkit_gb300.beams import make_beam
    rng = np.random.default_rng(7)
    t = 6 * 4 * 2 * 2
    ym = np.exp(rng.uniform(np.log(1e5), np.log(1e7), size=t))
    b = make_beam(4, 2, 2, ym=ym, pr=0.45, jitter=0.1, seed=11)
    J = ref["deformation_jacobian"](b.X, b.T)
    vol = ref["volume"](b.X, b.T)
    M = ref["massmatrix"](b.X, b.T, b.rho)
    x = b.X + 0.002 * rng.standard_normal(b.X.shape)
    s = ref["snh"]
    E = s.stable_neo_hookean_energy_x(x, J, b.mu, b.lam, vol)
    g = s.stable_neo_hookean_gradient_x(x, J, b.mu, b.lam, vol)
    K = s.stable_neo_hookean_hessian_x(x, J, b.mu, b.lam, vol).tocsr()
    K.sort_indices()
    np.savez_compressed(out, X=b.X, T=b.T, mu=b.mu, lam=b.lam, x=x,
                        J_data=J.data, J_indices=J.indices, J_indptr=J.indptr, J_shape=np.array(J.shape),
                        vol=vol, mass=M.diagonal(), energy=np.array(E), gradient=g,
                        K_data=K.data, K_indices=K.indices, K_indptr=K.indptr)


def make_beam_u_tier(ref, out):
    """simkit's *_u functions: stable_neo_hookean (snh.py:544-648) and the elastic dispatch
    (elastic.py:151-746) for the three other materials."""
    from simkit.energies import elastic as ref_elastic
    from simkit_gb300.beams import make_beam
    rng = np.random.default_rng(19)
    t = 6 * 3 * 2 * 2
    ym = np.exp(rng.uniform(np.log(1e5), np.log(1e7), size=t))
    b = make_beam(3, 2, 2, ym=ym, pr=0.42, jitter=0.1, seed=13)
    J = ref["deformation_jacobian"](b.X, b.T)
    vol = ref["volume"](b.X, b.T)
    x_bar = b.X + 0.01 * rng.standard_normal(b.X.shape)
    Jx_bar = J @ x_bar.reshape(-1, 1)
    u = 0.003 * rng.standard_normal(b.X.shape)
    s = ref["snh"]
    res = dict(X=b.X, T=b.T, mu=b.mu, lam=b.lam, vol=vol, u=u, Jx_bar=Jx_bar)
    res["snh_energy"] = np.array(s.stable_neo_hookean_energy_u(u, J, Jx_bar, b.mu, b.lam, vol))
    res["snh_gradient"] = s.stable_neo_hookean_gradient_u(u, J, Jx_bar, b.mu, b.lam, vol)
    res["snh_hessian"] = s.stable_neo_hookean_hessian_u(u, J, Jx_bar, b.mu, b.lam, vol).toarray()
    res["snh_hessian_raw"] = s.stable_neo_hookean_hessian_u(u, J, Jx_bar, b.mu, b.lam, vol, psd=False).toarray()
    for tag, mat in (("mmnh", "macklin-mueller-neo-hookean"), ("arap", "arap"), ("fcr", "fcr"),
                     ("le", "linear-elasticity")):
        res[f"{tag}_energy"] = np.array(ref_elastic.elastic_energy_u(u, J, Jx_bar, b.mu, b.lam, vol, mat))
        res[f"{tag}_gradient"] = ref_elastic.elastic_gradient_u(u, J, Jx_bar, b.mu, b.lam, vol, mat)
        res[f"{tag}_hessian"] = ref_elastic.elastic_hessian_u(u, J, Jx_bar, b.mu, b.lam, vol, mat).toarray()
        res[f"{tag}_hessian_raw"] = ref_elastic.elastic_hessian_u(u, J, Jx_bar, b.mu, b.lam, vol, mat,
                                                                  psd=False).toarray()
    np.savez_compressed(out, **res)


def make_contact_plane(ref, out):
    import scipy.sparse as sps
    rng = np.random.default_rng(21)
    X = rng.uniform(-1.0, 1.0, size=(200, 3))
    m = rng.uniform(0.5, 2.0, size=200)
    p = np.array([0.1, -0.2, 0.05])
    n = np.array([0.2, 1.0, -0.3])
    n = n / np.linalg.norm(n)
    k = 370.0
    c = ref["contact"]
    out_d = {}
    for tag, M in (("m", sps.diags(m)), ("i", None)):
        e, inds = c.contact_springs_plane_energy(X, k, p, n, M=M, return_contact_inds=True)
        g = c.contact_springs_plane_gradient(X, k, p, n, M=M)
        H = c.contact_springs_plane_hessian(X, k, p, n, M=M).tocsr()
        H.sort_indices()
        out_d.update({f"energy_{tag}": np.array(e), f"grad_{tag}": g, f"inds_{tag}": inds,
                      f"H_{tag}": H.toarray()})
    np.savez_compressed(out, X=X, m=m, p=p, n=n, k=k, **out_d)


def _reference_rollout(ref, spec, dt, steps, keep=None, integrator="be", material="snh", planes=None):
    """The oracle harness with every FEM routine and the Newton step taken from the reference."""
    import scipy.sparse as sps
    from oracle.rollout import BeamRollout

    if material == "mmnh":
        m = ref["mmnh"]
        s = type("MMNH", (), dict(
            stable_neo_hookean_energy_x=staticmethod(m.macklin_mueller_neo_hookean_energy_x),
            stable_neo_hookean_gradient_x=staticmethod(m.macklin_mueller_neo_hookean_gradient_x),
            stable_neo_hookean_hessian_x=staticmethod(m.macklin_mueller_neo_hookean_hessian_x)))
    elif material == "arap":
        a = ref["arap"]   # arap_*_x take no lam
        s = type("ARAP", (), dict(
            stable_neo_hookean_energy_x=staticmethod(lambda x, J, mu, lam, vol: a.arap_energy_x(x, J, mu, vol)),
            stable_neo_hookean_gradient_x=staticmethod(lambda x, J, mu, lam, vol: a.arap_gradient_x(x, J, mu, vol)),
            stable_neo_hookean_hessian_x=staticmethod(lambda x, J, mu, lam, vol: a.arap_hessian_x(x, J, mu, vol))))
    elif material == "le":
        m = ref["le"]
        s = type("LE", (), dict(
            stable_neo_hookean_energy_x=staticmethod(m.linear_elasticity_energy_x),
            stable_neo_hookean_gradient_x=staticmethod(m.linear_elasticity_gradient_x),
            stable_neo_hookean_hessian_x=staticmethod(m.linear_elasticity_hessian_x)))
    elif material == "fcr":
        f = ref["fcr"]
        s = type("FCR", (), dict(
            stable_neo_hookean_energy_x=staticmethod(f.fcr_energy_x),
            stable_neo_hookean_gradient_x=staticmethod(f.fcr_gradient_x),
            stable_neo_hookean_hessian_x=staticmethod(f.fcr_hessian_x)))
    else:
        s = ref["snh"]

    class RefRollout(BeamRollout):
        def __init__(self):
            super().__init__(spec.X, spec.T, spec.mu, spec.lam, spec.rho, spec.gravity,
                             spec.pinned, dt)
            self.J = ref["deformation_jacobian"](self.X, self.T)
            self.vol = ref["volume"](self.X, self.T)
            m = np.asarray(ref["massmatrix"](self.X, self.T, spec.rho).diagonal())
            self.mass = m
            self.f_ext = (m[:, None] * spec.gravity[None, :]).reshape(-1, 1)
            self.M = sps.diags(np.repeat(m, 3)).tocsc()
            self.Mf = (self.S @ self.M @ self.S.T).tocsc()

        def potential(self, x):
            e = s.stable_neo_hookean_energy_x(x.reshape(-1, 3), self.J, self.mu, self.lam, self.vol) \
                - (self.f_ext.T @ x).item()
            return e + (self.contact_energy(x) if self.planes else 0.0)

        def potential_gradient(self, x):
            g = s.stable_neo_hookean_gradient_x(x.reshape(-1, 3), self.J, self.mu, self.lam, self.vol) \
                - self.f_ext
            return g + self.contact_gradient(x) if self.planes else g

        def potential_hessian(self, x):
            K = s.stable_neo_hookean_hessian_x(x.reshape(-1, 3), self.J, self.mu, self.lam, self.vol)
            return (K + self.contact_hessian(x)).tocsr() if self.planes else K

        def elastic_energy(self, x):
            return s.stable_neo_hookean_energy_x(x.reshape(-1, 3), self.J, self.mu, self.lam, self.vol)

        def contact_energy(self, x):
            return sum(float(ref["contact"].contact_springs_plane_energy(x.reshape(-1, 3), k, p, n, M=self._contact_M()))
                       for k, p, n in self.planes)

        def contact_gradient(self, x):
            return sum(ref["contact"].contact_springs_plane_gradient(x.reshape(-1, 3), k, p, n, M=self._contact_M())
                       for k, p, n in self.planes)

        def contact_hessian(self, x):
            return sum(ref["contact"].contact_springs_plane_hessian(x.reshape(-1, 3), k, p, n, M=self._contact_M())
                       for k, p, n in self.planes)

        def be_target(self, yc, yp, h):
            return ref["kinetic"].be_target(yc, yp, h)

        def bdf2_target(self, yc, yp, yp2, yp3, h):
            return ref["kinetic"].bdf2_target(yc, yp, yp2, yp3, h)

    r = RefRollout()
    r.planes = list(planes or [])
    r.contact_mass_weighted = True
    assert ref["kinetic"]._BDF2_COEFF == 9.0 / 4.0
    x_prev3 = r.x_rest.copy()
    x_prev2 = r.x_rest.copy()
    x_prev = r.x_rest.copy()
    x_curr = r.x_rest.copy()
    us, energies, iters, res_last = {}, [], [], []
    for k in range(steps):
        if integrator == "bdf2":
            x_next, info = r.step(x_curr, x_prev, newton=ref["newton_solver"], x_prev2=x_prev2, x_prev3=x_prev3)
        else:
            x_next, info = r.step(x_curr, x_prev, newton=ref["newton_solver"])
        x_prev3, x_prev2, x_prev, x_curr = x_prev2, x_prev, x_curr, x_next
        energies.append(r.elastic_energy(x_curr))
        iters.append(info.iters)
        res_last.append(info.residuals[-1])
        if keep is None or (k + 1) in keep:
            us[k + 1] = (x_curr - r.x_rest).ravel()
    return us, np.array(energies), np.array(iters), np.array(res_last)


def make_rollout_small(ref, out):
    from simkit_gb300.beams import make_beam
    spec = make_beam(6, 2, 2, ym=2e5, pr=0.45)
    us, en, it, rl = _reference_rollout(ref, spec, 1.0 / 60.0, 8)
    keys = sorted(us)
    np.savez_compressed(out, steps=np.array(keys), u=np.stack([us[k] for k in keys]),
                        energy=en, iters=it, residual=rl, dims=np.array(spec.dims),
                        ym=2e5, pr=0.45, dt=1.0 / 60.0)


def make_rollout_bdf2_small(ref, out):
    from simkit_gb300.beams import make_beam
    spec = make_beam(6, 2, 2, ym=2e5, pr=0.45)
    us, en, it, rl = _reference_rollout(ref, spec, 1.0 / 60.0, 8, integrator="bdf2")
    keys = sorted(us)
    np.savez_compressed(out, steps=np.array(keys), u=np.stack([us[k] for k in keys]),
                        energy=en, iters=it, residual=rl, dims=np.array(spec.dims),
                        ym=2e5, pr=0.45, dt=1.0 / 60.0)


def make_rollout_mmnh_small(ref, out):
    from simkit_gb300.beams import make_beam
    spec = make_beam(6, 2, 2, ym=2e5, pr=0.45)
    us, en, it, rl = _reference_rollout(ref, spec, 1.0 / 60.0, 8, material="mmnh")
    keys = sorted(us)
    np.savez_compressed(out, steps=np.array(keys), u=np.stack([us[k] for k in keys]),
                        energy=en, iters=it, residual=rl, dims=np.array(spec.dims),
                        ym=2e5, pr=0.45, dt=1.0 / 60.0)


def make_rollout_corot_small(ref, out, material):
    from simkit_gb300.beams import make_beam
    spec = make_beam(6, 2, 2, ym=2e5, pr=0.45)
    us, en, it, rl = _reference_rollout(ref, spec, 1.0 / 60.0, 8, material=material)
    keys = sorted(us)
    np.savez_compressed(out, steps=np.array(keys), u=np.stack([us[k] for k in keys]),
                        energy=en, iters=it, residual=rl, dims=np.array(spec.dims),
                        ym=2e5, pr=0.45, dt=1.0 / 60.0)


FLOOR = (1.0e4, (0.0, -0.004, 0.0), (0.0, 1.0, 0.0))   # k (mass weighted), point, normal


def make_rollout_contact_small(ref, out):
    from simkit_gb300.beams import make_beam
    spec = make_beam(6, 2, 2, ym=2e5, pr=0.45)
    planes = [(FLOOR[0], np.array(FLOOR[1]), np.array(FLOOR[2]))]
    us, en, it, rl = _reference_rollout(ref, spec, 1.0 / 60.0, 14, material="mmnh", planes=planes)
    keys = sorted(us)
    np.savez_compressed(out, steps=np.array(keys), u=np.stack([us[k] for k in keys]),
                        energy=en, iters=it, residual=rl, dims=np.array(spec.dims),
                        ym=2e5, pr=0.45, dt=1.0 / 60.0, k=FLOOR[0], p=np.array(FLOOR[1]), n=np.array(FLOOR[2]))


def make_cache_file(ref_path, out):
    sys.path.insert(0, ref_path)
    from simkit.filesystem.compute_with_cache_check import compute_with_cache_check
    if os.path.exists(out):
        os.remove(out)
    rng = np.random.default_rng(31)
    traj = rng.standard_normal((3, 5, 3))
    compute_with_cache_check(lambda: (traj, 7, np.array([2.5]), np.arange(4)), out, read_cache=False)


def make_rollout_c1(ref, out):
    from simkit_gb300.beams import beam_small_steady
    spec = beam_small_steady()
    keep = (1, 2, 5, 10, 20, 30, 45, 60)
    t0 = time.time()
    us, en, it, rl = _reference_rollout(ref, spec, 1.0 / 60.0, 60, keep=keep)
    print(f"  reference 8x8x32 rollout: {time.time() - t0:.1f} s, {it.sum()} Newton iterations")
    keys = sorted(us)
    np.savez_compressed(out, steps=np.array(keys), u=np.stack([us[k] for k in keys]),
                        energy=en, iters=it, residual=rl, dt=1.0 / 60.0)


class _TightPCG:
    """A stand-in for ``scipy.sparse.linalg.spsolve`` on the free-DOF Hessians of one beam: CG to a
    1e-10 relative residual, preconditioned by 3x3 block Jacobi plus a rigid-mode coarse space (six
    modes per box of 8^3 cells, Cholesky of P^T A P).  On the 786,432-tet beam simkit's own call
    (SuperLU) did not finish in 25 minutes; this solve agrees with an exact one to the 1e-10
    residual, far below the 1e-6 Newton tolerance the rollout stops at."""

    def __init__(self, X_free_verts, cell, box=8, rtol=1e-10, max_iter=20000):
        import scipy.sparse as sps
        Xv = np.asarray(X_free_verts, dtype=np.float64)
        nv = Xv.shape[0]
        key = np.floor(Xv / (box * cell) + 1e-9).astype(np.int64)
        _, agg = np.unique(key, axis=0, return_inverse=True)
        agg = agg.ravel()
        na = int(agg.max()) + 1
        cnt = np.bincount(agg, minlength=na).astype(np.float64)
        cen = np.stack([np.bincount(agg, weights=Xv[:, k], minlength=na) for k in range(3)], 1) / cnt[:, None]
        d = Xv - cen[agg]
        rms = np.sqrt(np.bincount(agg, weights=(d * d).sum(1), minlength=na) / cnt) + 1e-30
        d = d / rms[agg][:, None]
        rows, cols, vals = [], [], []
        v = np.arange(nv)
        for c in range(3):                                # translations
            rows.append(3 * v + c); cols.append(6 * agg + c); vals.append(np.ones(nv))
        # rotations w x d: row x gets (w_y d_z - w_z d_y), y gets (w_z d_x - w_x d_z), z (w_x d_y - w_y d_x)
        for r, (ca, sa), (cb, sb) in ((0, (4, 2), (5, 1)), (1, (5, 0), (3, 2)), (2, (3, 1), (4, 0))):
            rows.append(3 * v + r); cols.append(6 * agg + ca); vals.append(d[:, sa])
            rows.append(3 * v + r); cols.append(6 * agg + cb); vals.append(-d[:, sb])
        P = sps.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                           shape=(3 * nv, 6 * na))
        # aggregates of one vertex (or of collinear vertices) give zero rotation columns: drop them
        norms = np.sqrt(np.asarray(P.multiply(P).sum(axis=0)).ravel())
        self.P = P[:, norms > 1e-9 * norms.max()].tocsr()
        self.nv, self.rtol, self.max_iter = nv, rtol, max_iter
        self.worst = 0.0
        self.iters = []

    def __call__(self, A, b):
        import scipy.linalg as sla
        A = A.tocsr()
        n = A.shape[0]
        assert n == 3 * self.nv
        b = np.asarray(b, dtype=np.float64).reshape(-1)
        # 3x3 diagonal blocks
        D = np.zeros((self.nv, 3, 3))
        Ac = A.tocoo()
        on = (Ac.row // 3) == (Ac.col // 3)
        np.add.at(D, (Ac.row[on] // 3, Ac.row[on] % 3, Ac.col[on] % 3), Ac.data[on])
        Dinv = np.linalg.inv(D)
        Acoarse = (self.P.T @ (A @ self.P)).toarray()
        Acoarse[np.diag_indices_from(Acoarse)] *= 1.0 + 1e-10    # linearly dependent modes stay invertible
        cf = sla.cho_factor(Acoarse)
        P = self.P

        def prec(r):
            z = np.einsum("vij,vj->vi", Dinv, r.reshape(-1, 3)).reshape(-1)
            return z + P @ sla.cho_solve(cf, P.T @ r)

        x = np.zeros(n)
        r = b.copy()
        bn = np.linalg.norm(b)
        z = prec(r)
        p = z.copy()
        rz = r @ z
        it = 0
        while np.linalg.norm(r) > self.rtol * bn and it < self.max_iter:
            q = A @ p
            a = rz / (p @ q)
            x += a * p
            r -= a * q
            z = prec(r)
            rz_new = r @ z
            p = z + (rz_new / rz) * p
            rz = rz_new
            it += 1
        rel = float(np.linalg.norm(b - A @ x) / bn)
        assert rel < 10 * self.rtol, f"PCG stalled at {rel:.2e}"
        self.worst = max(self.worst, rel)
        self.iters.append(it)
        return x


def make_rollout_c2_first_steps(ref, out, steps=2, stride=8):
    """The benchmarked 786,432-tet beam (32x32x128 cubes, rest shape jittered by U(-0.1, 0.1) cells,
    E log-uniform [1e5, 1e7] per tet, seed 0): the first ``steps`` backward-Euler steps from rest with
    simkit's energies, Hessians (incl. psd_project), line search and newton_solver, under the harness
    rules of oracle/rollout.py.  The one substitution: simkit's ``spsolve`` is replaced by a PCG to a
    1e-10 relative residual (_TightPCG) because SuperLU does not finish on this mesh.  Stored: the
    displacement of every ``stride``-th vertex and of every vertex on the free end face, per step."""
    import scipy.sparse.linalg as spla
    from simkit_gb300.beams import beam_large_jittered
    spec = beam_large_jittered(seed=0)
    n = spec.n_verts
    pin = np.zeros(n, bool)
    pin[spec.pinned] = True
    solver = _TightPCG(spec.X[~pin], cell=0.025)
    tip = np.nonzero(np.isclose(spec.X[:, 0], spec.X[:, 0].max()))[0]
    sample = np.union1d(np.arange(0, n, stride), tip)
    orig = spla.spsolve
    spla.spsolve = solver
    t0 = time.time()
    try:
        us, en, it, rl = _reference_rollout(ref, spec, 1.0 / 60.0, steps)
    finally:
        spla.spsolve = orig
    print(f"  reference 32x32x128 first {steps} steps: {time.time() - t0:.1f} s, Newton iterations {list(it)}, "
          f"PCG iterations {solver.iters}, worst solve residual {solver.worst:.2e}")
    keys = sorted(us)
    U = np.stack([us[k].reshape(-1, 3)[sample] for k in keys])
    np.savez_compressed(out, steps=np.array(keys), sample=sample, u=U, energy=en, iters=it, residual=rl,
                        dims=np.array(spec.dims), seed=0, dt=1.0 / 60.0, solve_rtol=solver.rtol,
                        solve_worst=solver.worst, solve_iters=np.array(solver.iters),
                        solve="PCG (3x3 block Jacobi + rigid-mode aggregates of 8^3 cells) to 1e-10 relative "
                              "residual in place of scipy spsolve")


def _write_corot(ref):
    for mat in ("arap", "fcr"):
        make_element_corot(ref, 3, os.path.join(HERE, f"element_{mat}_3d.npz"), mat)
        make_element_corot(ref, 2, os.path.join(HERE, f"element_{mat}_2d.npz"), mat)
        make_rollout_corot_small(ref, os.path.join(HERE, f"rollout_{mat}_small.npz"), mat)


def _write_le(ref):
    make_element_le(ref, 3, os.path.join(HERE, "element_le_3d.npz"))
    make_element_le(ref, 2, os.path.join(HERE, "element_le_2d.npz"))
    make_rollout_corot_small(ref, os.path.join(HERE, "rollout_le_small.npz"), "le")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("SIMKIT_REFERENCE"),
                    help="path of a simkit checkout (or set SIMKIT_REFERENCE)")
    ap.add_argument("--skip-c1", action="store_true")
    ap.add_argument("--skip-c2", action="store_true")
    ap.add_argument("--only", default="", help="comma-separated groups to (re)write: corot, le, u, c2")
    a = ap.parse_args()
    if not a.reference:
        ap.error("give --reference or set SIMKIT_REFERENCE to a simkit checkout")
    ref = _import_reference(a.reference)
    if a.only:
        if "c2" in a.only.split(","):
            make_rollout_c2_first_steps(ref, os.path.join(HERE, "rollout_beam_32x32x128_first_steps.npz"))
        if "corot" in a.only.split(","):
            _write_corot(ref)
        if "le" in a.only.split(","):
            _write_le(ref)
        if "u" in a.only.split(","):
            make_beam_u_tier(ref, os.path.join(HERE, "beam_u_tier.npz"))
        print("fixtures written to", HERE)
        return
    make_element(ref, 3, os.path.join(HERE, "element_3d.npz"))
    make_element(ref, 2, os.path.join(HERE, "element_2d.npz"))
    make_beam_small(ref, os.path.join(HERE, "beam_small.npz"))
    make_rollout_small(ref, os.path.join(HERE, "rollout_small.npz"))
    make_rollout_bdf2_small(ref, os.path.join(HERE, "rollout_bdf2_small.npz"))
    make_element_mmnh(ref, 3, os.path.join(HERE, "element_mmnh_3d.npz"))
    make_element_mmnh(ref, 2, os.path.join(HERE, "element_mmnh_2d.npz"))
    make_rollout_mmnh_small(ref, os.path.join(HERE, "rollout_mmnh_small.npz"))
    make_contact_plane(ref, os.path.join(HERE, "contact_plane.npz"))
    make_rollout_contact_small(ref, os.path.join(HERE, "rollout_contact_small.npz"))
    make_cache_file(a.reference, os.path.join(HERE, "cache_reference.npz"))
    _write_corot(ref)
    _write_le(ref)
    make_beam_u_tier(ref, os.path.join(HERE, "beam_u_tier.npz"))
    if not a.skip_c1:
        make_rollout_c1(ref, os.path.join(HERE, "rollout_beam_8x8x32.npz"))
    if not a.skip_c2:
        make_rollout_c2_first_steps(ref, os.path.join(HERE, "rollout_beam_32x32x128_first_steps.npz"))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
