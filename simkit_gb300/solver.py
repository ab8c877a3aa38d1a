"""Device-resident backward-Euler rollout of one elastic body.

``BESolver.step()`` is one call of simkit's ``backward_euler`` (
``simkit/integrators/backward_euler.py:27-91``) with the stable neo-Hookean
closures, gravity, pinned DOFs held at rest, and Newton iterated until the
relative residual ``||g(x)|| / ||g(x_tilde)||`` falls below ``tol`` - all on
the GPU through ``skg_be_step`` (or its recorded graph, ``skg_be_plan_*``).  Positions
stay in HBM between steps.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import BEParamsC, BEStateC, StepInfoC, check, SKG_FP64, SKG_MIXED
from .mesh import TetMesh, _stream_ptr

PRECISIONS = {"fp64": SKG_FP64, "mixed": SKG_MIXED}
INTEGRATORS = {"be": 0, "bdf2": 1}


@dataclass
class StepInfo:
    newton_iters: int
    pcg_iters: int
    ls_trials: int
    status: int
    residual0: float
    residual: float
    min_alpha: float
    energy: float
    launches: int = 0
    t_hessian_ms: float = 0.0
    t_assemble_ms: float = 0.0
    t_pcg_ms: float = 0.0
    t_gradient_ms: float = 0.0
    t_energy_ms: float = 0.0
    warm_used: int = 0

    @property
    def converged(self) -> bool:
        return self.status == 0


def tet_volumes_host(X, T) -> np.ndarray:
    """Signed tet volumes (X1-X0) . ((X2-X0) x (X3-X0)) / 6 (simkit/volume.py:14-41)."""
    a, b, c = (X[T[:, k]] - X[T[:, 0]] for k in (1, 2, 3))
    det = (a[:, 0] * (b[:, 1] * c[:, 2] - b[:, 2] * c[:, 1]) - a[:, 1] * (b[:, 0] * c[:, 2] - b[:, 2] * c[:, 0])
           + a[:, 2] * (b[:, 0] * c[:, 1] - b[:, 1] * c[:, 0]))
    return det / 6.0


def lumped_mass(X, T, rho) -> np.ndarray:
    """sum over incident tets of rho vol / 4 (simkit/massmatrix.py:40-50), in tet order."""
    T = np.asarray(T)
    vol = tet_volumes_host(np.asarray(X, dtype=np.float64), T)
    w = np.repeat(np.asarray(rho, dtype=np.float64) * vol / 4.0, 4)
    return np.bincount(T.ravel(), weights=w, minlength=X.shape[0])


class BESolver:
    """Backward-Euler stepper for one tet mesh on one GPU.

    Parameters
    ----------
    X, T, mu, lam : rest mesh and per-tet Lame parameters (simkit conventions)
    rho : density; gravity : (3,) acceleration; pinned : vertex indices held at rest
    dt : time step; tol : relative residual stop; max_newton : Newton cap
    precision : 'mixed' (FP32 Hessian/SpMV, FP64 residual/dots/energy sums) or 'fp64'
    pcg_rtol : PCG relative tolerance; a negative value selects Eisenstat-Walker
        forcing capped at its magnitude
    pcg_mode : 0 kernel per phase, 1 grid-persistent, 2 one thread-block
        cluster, 3 choose by size (cluster up to 24,576 block rows, else 7 with coarse
        data, else 5), 5 grid-persistent with two barriers per iteration, 7 its two-level form
    integrator : 'be' (simkit/integrators/backward_euler.py) or 'bdf2'
        (simkit/integrators/bdf2.py: four displacement levels, all at rest initially)
    material : 'stable-neo-hookean', 'macklin-mueller-neo-hookean', 'arap', 'fcr' or
        'linear-elasticity' (simkit/energies/elastic.py names; 'arap' ignores lam)
    contact_planes : optional list of (k, p, n) contact-spring planes added to the potential
    coarse : two-level PCG preconditioner (block Jacobi + rigid-mode aggregates of box^3 mesh
        spacings): None (one-level), 'auto' or a box size.  Meshes above 24,576 vertices get the
        whole-mesh form (the grid PCG, pcg_mode 3 or 7; 'auto': the finest box from 6 spacings up
        whose coarse space fits 3,072 unknowns, box 7 on the 32 x 32 x 128 beam), smaller ones the
        per-instance form (box 4; the thread-block-cluster PCG, pcg_mode 2 or 3)
    coarse_form : 'auto' (by size, as above), 'grid' or 'cluster'
    mass, f_ext : per-vertex lumped masses (n) and external forces (3n) instead of the ones
        ``rho`` and ``gravity`` give
    coarse_refresh : 'step' (coarse inverse rebuilt at the first Newton iteration of each step),
        'newton' (at every Newton iteration) or an int k (default 4: at the first Newton iteration
        of every k-th step; the steps between reuse it: the preconditioner stays SPD, only less
        fresh, and on the 786,432-tet beam the PCG iteration count did not change)
    ew_gamma, ew_alpha : Eisenstat-Walker choice 2 (with pcg_rtol < 0), after the first Newton
        iteration eta = ew_gamma (r_k / r_{k-1})^ew_alpha, safeguarded; exponents in quarter steps
        over [1, 2] are evaluated alike on the host and the device.  On the 786,432-tet beam the
        Newton residual falls about as far as each linear solve's tolerance, so the exponent sets the
        trade of Newton iterations against PCG iterations: 1.25 (6.15 Newton, 164 PCG iterations
        per step) ran 80.6 steps/s, 2 (5.45, 207) 71.5
    device_loop : run each step as a recorded CUDA graph with the Newton loop and line search decided
        on the device (``skg_be_plan_*``: one host synchronisation per step instead of two per Newton
        iteration, bitwise the same steps) when the parameters allow it (the grid PCG forms; profiled
        steps, Newton records and simkit's stop rule take the host loop)
    """

    def __init__(self, X, T, mu, lam, rho=1000.0, gravity=(0.0, -9.8, 0.0), pinned=(), dt=1.0 / 60.0,
                 tol=1e-6, max_newton=20, precision="mixed", pcg_rtol=-0.1, pcg_max_iter=4000, pcg_mode=3,
                 do_line_search=True, ls_threshold=None, profile=False, device="cuda", integrator="be",
                 material="stable-neo-hookean", contact_planes=None, contact_mass_weighted=True,
                 coarse="auto", coarse_refresh=4, coarse_form="auto", mass=None, f_ext=None, device_loop=True,
                 ew_gamma=0.9, ew_alpha=1.25):
        _lib.load()
        self.mesh = TetMesh(X, T, mu, lam, device=device)
        self.mesh.check_orientation()
        self.mesh.set_energy(material)
        m = self.mesh
        dev = m.device
        X = m.X_host
        self.precision = PRECISIONS[precision]
        mass = lumped_mass(X, m.T_host, rho) if mass is None else np.asarray(mass, dtype=np.float64).reshape(-1)
        if mass.size != m.n:
            raise ValueError("mass needs one lumped value per vertex")
        self.mass = torch.from_numpy(mass).to(dev)
        if f_ext is None:
            g = np.asarray(gravity, dtype=np.float64)
            f_ext = (mass[:, None] * g[None, :]).reshape(-1)
        f_ext = np.asarray(f_ext, dtype=np.float64).reshape(-1)
        if f_ext.size != 3 * m.n:
            raise ValueError("f_ext needs 3 values per vertex")
        self.f_ext = torch.from_numpy(f_ext.copy()).to(dev)
        pin = np.zeros(3 * m.n, np.uint8)
        pv = np.asarray(pinned, dtype=np.int64).ravel()
        pin[(3 * pv[:, None] + np.arange(3)[None, :]).ravel()] = 1
        self.pinned = torch.from_numpy(pin).to(dev)
        self.coarse_box = None
        self.coarse_form = None
        if coarse is not None:
            form = coarse_form if coarse_form != "auto" else ("grid" if m.n > 24576 else "cluster")
            if form not in ("grid", "cluster"):
                raise ValueError("coarse_form must be 'auto', 'grid' or 'cluster'")
            self.coarse_form = form
            if form == "grid":
                _, self.coarse_box = m.set_coarse(pin == 0, box=None if coarse == "auto" else int(coarse))
            else:
                _, boxes = m.set_coarse_inst(pin == 0, box=4 if coarse == "auto" else int(coarse))
                self.coarse_box = int(boxes[0])
        if not (coarse_refresh in ("step", "newton") or (isinstance(coarse_refresh, int) and coarse_refresh >= 1)):
            raise ValueError("coarse_refresh must be 'step', 'newton' or an int >= 1")
        self.coarse_refresh = coarse_refresh
        self._coarse_age = None   # steps since the coarse inverse was built (None: not built)
        self.u_prev = torch.zeros(3 * m.n, dtype=torch.float64, device=dev)
        self.u_curr = torch.zeros_like(self.u_prev)
        self.u_next = torch.zeros_like(self.u_prev)
        if integrator not in INTEGRATORS:
            raise ValueError(f"integrator must be one of {sorted(INTEGRATORS)}")
        self.integrator = integrator
        self.u_prev2 = torch.zeros_like(self.u_prev) if integrator == "bdf2" else None
        self.u_prev3 = torch.zeros_like(self.u_prev) if integrator == "bdf2" else None
        nbytes = _lib.load().skg_be_workspace_size(ctypes.byref(m.c), self.precision)
        if nbytes < 0:
            raise ValueError(_lib.last_error())
        self.workspace = torch.zeros(int(nbytes), dtype=torch.uint8, device=dev)
        self.params = BEParamsC(
            dt=dt, tol=tol, max_newton=max_newton, precision=self.precision, pcg_rtol=pcg_rtol,
            pcg_max_iter=pcg_max_iter, do_line_search=int(do_line_search), ls_alpha=0.01, ls_beta=0.5,
            ls_max_iter=100, pcg_mode=pcg_mode,
            ls_threshold=(-1.0 if precision == "mixed" else 1e-12) if ls_threshold is None else ls_threshold,
            profile=int(profile), integrator=INTEGRATORS[integrator],
            coarse_refresh=int(coarse_refresh == "newton"), ew_gamma=ew_gamma, ew_alpha=ew_alpha)
        self.set_contact_planes(contact_planes, contact_mass_weighted)
        self.steps = 0
        self._host = None
        self.device_loop = bool(device_loop)
        self._plans = {}          # device-loop graphs, one per rotation of the state buffers and refresh flag
        self._plan_key = None     # parameters, contact planes and mesh arrays the plans were recorded with
        self._eligible = None     # (key, whether those parameters can be recorded)

    def _coarse_n_agg(self) -> int:
        return int(self.mesh._coarse_c.n_agg) if getattr(self.mesh, "_coarse_c", None) is not None else 0

    def refresh_coarse(self):
        """Rebuild the coarse inverse at the next step's first Newton iteration (and count the refresh
        period from there)."""
        self._coarse_age = None

    def set_contact_planes(self, planes, mass_weighted=True):
        """Contact springs against planes, each (k, p, n) (simkit/energies/contact_springs_plane.py);
        mass_weighted: spring weights are the lumped vertex masses (simkit's M) instead of 1."""
        self._planes, n = _lib.contact_planes(planes)
        self.params.n_planes = n
        self.params.contact_mass_weighted = int(bool(mass_weighted))
        self.params.planes = ctypes.cast(self._planes, ctypes.POINTER(_lib.ContactPlaneC))

    @classmethod
    def from_spec(cls, spec, **kw):
        return cls(spec.X, spec.T, spec.mu, spec.lam, rho=spec.rho, gravity=spec.gravity, pinned=spec.pinned, **kw)

    def _state(self):
        bdf2 = self.integrator == "bdf2"
        return BEStateC(u=self.u_next.data_ptr(), u_curr=self.u_curr.data_ptr(), u_prev=self.u_prev.data_ptr(),
                        mass=self.mass.data_ptr(), f_ext=self.f_ext.data_ptr(), pinned=self.pinned.data_ptr(),
                        u_prev2=self.u_prev2.data_ptr() if bdf2 else None,
                        u_prev3=self.u_prev3.data_ptr() if bdf2 else None, x_rest=self.mesh.X.data_ptr())

    def _rotate(self):
        """History after a step: [prev3 <- prev2 <-] prev <- curr <- next (next becomes scratch)."""
        if self.integrator == "bdf2":
            self.u_prev3, self.u_prev2, self.u_prev, self.u_curr, self.u_next = (
                self.u_prev2, self.u_prev, self.u_curr, self.u_next, self.u_prev3)
        else:
            self.u_prev, self.u_curr, self.u_next = self.u_curr, self.u_next, self.u_prev

    def prepare_plans(self) -> int:
        """Record now the device-loop graphs of every rotation of the state buffers and both coarse
        refresh decisions, so that no later step records one; returns how many exist (0 when the
        parameters take the host loop)."""
        if not self.device_loop:
            return 0
        rotations = 5 if self.integrator == "bdf2" else 3
        flags = (0, -1) if isinstance(self.coarse_refresh, int) else (self.params.coarse_refresh,)
        keep = self.params.coarse_refresh
        try:
            for _ in range(rotations):
                for f in flags:
                    self.params.coarse_refresh = f
                    if self._plan(self._state()) is None:
                        return 0
                self._rotate()
        finally:
            self.params.coarse_refresh = keep
        return len(self._plans)

    def step(self, stream=None) -> StepInfo:
        st = self._state()
        info = StepInfoC()
        if isinstance(self.coarse_refresh, int):
            rebuild = self._coarse_age is None or self._coarse_age + 1 >= self.coarse_refresh
            self.params.coarse_refresh = 0 if rebuild else -1
            self._coarse_age = 0 if rebuild else self._coarse_age + 1
        plan = self._plan(st) if self.device_loop else None
        if plan is not None:
            check(_lib.load().skg_be_plan_step(plan, ctypes.byref(info), _stream_ptr(stream)))
        else:
            check(_lib.load().skg_be_step(ctypes.byref(self.mesh.c), ctypes.byref(self.params), ctypes.byref(st),
                                          ctypes.c_void_p(self.workspace.data_ptr()), ctypes.byref(info),
                                          _stream_ptr(stream)))
        self._rotate()
        self.steps += 1
        return StepInfo(info.newton_iters, info.pcg_iters, info.ls_trials, info.status, info.residual0,
                        info.residual, info.min_alpha, info.energy, info.launches, info.t_hessian_ms,
                        info.t_assemble_ms, info.t_pcg_ms, info.t_gradient_ms, info.t_energy_ms)

    def _params_key(self):
        """What the device-loop graphs depend on besides the state buffers: the parameters (less the
        per-step refresh decision: graphs for both decisions are kept), the contact planes and the
        mesh's device arrays."""
        refresh = self.params.coarse_refresh
        self.params.coarse_refresh = 0
        raw = ctypes.string_at(ctypes.addressof(self.params), ctypes.sizeof(self.params))
        self.params.coarse_refresh = refresh
        planes = ctypes.string_at(ctypes.addressof(self._planes), ctypes.sizeof(self._planes)) if self._planes else b""
        mesh = ctypes.string_at(ctypes.addressof(self.mesh.c), ctypes.sizeof(self.mesh.c))
        coarse = getattr(self.mesh, "_coarse_c", None)
        cbytes = ctypes.string_at(ctypes.addressof(coarse), ctypes.sizeof(coarse)) if coarse is not None else b""
        return raw + planes + mesh + cbytes

    def _plan(self, st):
        """The device-loop graph for this state binding and refresh decision (recorded on first use, all
        of them again after a change of the parameters, planes or mesh arrays), or None when the
        parameters need the host loop (profiling, a Newton record, simkit's stop rule, the cluster PCG
        of small meshes)."""
        key = self._params_key()
        if self._eligible is None or self._eligible[0] != key:
            ok = bool(_lib.load().skg_be_plan_eligible(ctypes.byref(self.mesh.c), ctypes.byref(self.params)))
            self._eligible = (key, ok)
        if not self._eligible[1]:
            return None
        if key != self._plan_key:
            self.release_plans()
            self._plan_key = key
        bind = (st.u, st.u_curr, st.u_prev, st.u_prev2, st.u_prev3, self.params.coarse_refresh)
        plan = self._plans.get(bind)
        if plan is None:
            h = ctypes.c_void_p()
            check(_lib.load().skg_be_plan_create(ctypes.byref(self.mesh.c), ctypes.byref(self.params),
                                                 ctypes.byref(st), ctypes.c_void_p(self.workspace.data_ptr()),
                                                 ctypes.byref(h)))
            plan = self._plans[bind] = h
        return plan

    def release_plans(self):
        for h in getattr(self, "_plans", {}).values():
            _lib.load().skg_be_plan_destroy(h)
        self._plans = {}

    def __del__(self):
        try:
            self.release_plans()
        except Exception:
            pass

    def step_host(self, x_curr: np.ndarray, x_prev: np.ndarray, out: np.ndarray = None, stream=None,
                  x_prev2: np.ndarray = None, x_prev3: np.ndarray = None):
        """One step with host positions in and out (simkit's backward_euler contract:
        x_curr, x_prev (3n, 1) float64 -> x_next).  Copies the caller's arrays straight to the
        device and the result straight into ``out`` (no intermediate host copy: a DMA when the
        arrays live in pinned memory, the driver's pageable path otherwise).  A BDF2 solver also
        takes the positions two and three steps back (simkit's bdf2 contract)."""
        m = self.mesh
        if self._host is None:
            self._host = True
            self._X = torch.from_numpy(m.X_host.reshape(-1).copy()).to(m.device)
        xc = torch.from_numpy(np.ascontiguousarray(x_curr, dtype=np.float64).reshape(-1))
        xp = torch.from_numpy(np.ascontiguousarray(x_prev, dtype=np.float64).reshape(-1))
        self.u_curr.copy_(xc, non_blocking=xc.is_pinned())
        self.u_prev.copy_(xp, non_blocking=xp.is_pinned())
        self.u_curr.sub_(self._X)
        self.u_prev.sub_(self._X)
        if self.integrator == "bdf2":
            if x_prev2 is None or x_prev3 is None:
                raise ValueError("a BDF2 step needs x_prev2 and x_prev3")
            for dst, src in ((self.u_prev2, x_prev2), (self.u_prev3, x_prev3)):
                t = torch.from_numpy(np.ascontiguousarray(src, dtype=np.float64).reshape(-1))
                dst.copy_(t, non_blocking=t.is_pinned())
                dst.sub_(self._X)
        info = self.step(stream)
        self.u_next.copy_(self.u_curr).add_(self._X)      # u_next is scratch after the rotation
        if out is not None and out.dtype == np.float64 and out.flags["C_CONTIGUOUS"] and out.size == 3 * m.n:
            torch.from_numpy(out.reshape(-1)).copy_(self.u_next)   # synchronous device->host
            return out, info
        res = np.empty((3 * m.n, 1), dtype=np.float64)
        torch.from_numpy(res.reshape(-1)).copy_(self.u_next)
        if out is not None:
            out[...] = res
            return out, info
        return res, info

    def displacement(self) -> np.ndarray:
        return self.u_curr.cpu().numpy().copy()

    def positions(self) -> np.ndarray:
        return self.mesh.X_host.reshape(-1) + self.displacement()

    def set_state(self, u_curr, u_prev, u_prev2=None, u_prev3=None):
        """Displacement history (host or device arrays); the BDF2 levels k-2 and k-3 are
        needed with integrator 'bdf2'."""
        dev = lambda a: torch.as_tensor(np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a,
                                                   dtype=np.float64).reshape(-1))
        self.u_curr.copy_(dev(u_curr))
        self.u_prev.copy_(dev(u_prev))
        if self.integrator == "bdf2":
            if u_prev2 is None or u_prev3 is None:
                raise ValueError("BDF2 needs the displacements at steps k-2 and k-3")
            self.u_prev2.copy_(dev(u_prev2))
            self.u_prev3.copy_(dev(u_prev3))

    def rollout(self, steps, callback=None):
        infos = []
        for k in range(steps):
            info = self.step()
            infos.append(info)
            if callback is not None:
                callback(k, self, info)
        return infos
