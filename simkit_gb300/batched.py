"""Batched backward Euler: many independent meshes stepped together on one GPU.

simkit steps one mesh per ``backward_euler`` call
(``simkit/integrators/backward_euler.py:27-91``).  ``BatchedBESolver`` takes a
list of meshes of uneven sizes, concatenates them into one device mesh with
disjoint vertex and tet ranges, and advances all of them by one
backward-Euler step per call: the element, assembly and gradient kernels run
once over the concatenation, and every instance gets its own Newton
iteration, forcing term, Armijo search and convergence test, with its linear
system solved on a thread-block cluster taken from a largest-first queue.

By default a step is one launch of a CUDA graph with the Newton loop on the
device (``skg_be_batch_plan_*``: per-instance decisions in control kernels,
the Newton iterations and line-search trials as conditional graph nodes), one
plan per rotation of the state buffers; profiled steps and ``graph=False``
take ``skg_be_step_batched``, which makes the same decisions on the host.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import BatchC, BEParamsC, BEStateC, StepInfoC, check
from .mesh import TetMesh, _stream_ptr
from .solver import INTEGRATORS, PRECISIONS, StepInfo, lumped_mass


class BatchedBESolver:
    """Backward-Euler stepper for a batch of independent tet meshes.

    ``specs`` is a list of objects with ``X, T, mu, lam, rho, gravity,
    pinned`` (e.g. ``simkit_gb300.beams.BeamSpec``); each keeps its own
    material, gravity direction and pins.  ``coarse``: two-level PCG with
    per-instance aggregates ('auto': 4^3 mesh spacings, or a box size), None for
    the one-level block-Jacobi PCG; ``coarse_refresh``: 'step' (per-instance coarse inverses
    rebuilt at the first Newton iteration of each step), 'newton' (at every iteration) or an int k
    (at the first Newton iteration of every k-th step; the steps between reuse them).
    """

    def __init__(self, specs, dt=1.0 / 60.0, tol=1e-6, max_newton=20, precision="mixed", pcg_rtol=-0.1,
                 pcg_max_iter=4000, do_line_search=True, ls_threshold=None, profile=False, device="cuda",
                 integrator="be", material="stable-neo-hookean", contact_planes=None, contact_mass_weighted=True,
                 coarse="auto", coarse_refresh="step", graph=True, ew_gamma=0.9, ew_alpha=1.25):
        _lib.load()
        self.graph = graph
        self.n_inst = len(specs)
        if self.n_inst == 0:
            raise ValueError("empty batch")
        Xs, Ts, mus, lams, masses, fexts, pins = [], [], [], [], [], [], []
        rows, tets = [0], [0]
        for sp in specs:
            X = np.asarray(sp.X, dtype=np.float64).reshape(-1, 3)
            T = np.asarray(sp.T).reshape(-1, 4)
            Xs.append(X)
            Ts.append(T + rows[-1])
            mus.append(np.asarray(sp.mu, dtype=np.float64).reshape(-1))
            lams.append(np.asarray(sp.lam, dtype=np.float64).reshape(-1))
            m = lumped_mass(X, T, sp.rho)
            masses.append(m)
            fexts.append((m[:, None] * np.asarray(sp.gravity, dtype=np.float64)[None, :]).reshape(-1))
            p = np.zeros(3 * X.shape[0], np.uint8)
            pv = np.asarray(sp.pinned, dtype=np.int64).ravel()
            p[(3 * pv[:, None] + np.arange(3)[None, :]).ravel()] = 1
            pins.append(p)
            rows.append(rows[-1] + X.shape[0])
            tets.append(tets[-1] + T.shape[0])
        mesh = TetMesh(np.concatenate(Xs), np.concatenate(Ts), np.concatenate(mus), np.concatenate(lams),
                       device=device)
        mesh.check_orientation()
        mesh.set_energy(material)
        up = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(mesh.device)
        self._contact_init = (contact_planes, contact_mass_weighted)
        # two-level PCG: per-instance aggregates (box 4 mesh spacings by default)
        self.coarse_boxes = None
        if coarse is not None:
            _, self.coarse_boxes = mesh.set_coarse_inst(np.concatenate(pins) == 0, np.array(rows),
                                                        box=4 if coarse == "auto" else int(coarse))
        if not (coarse_refresh in ("step", "newton") or (isinstance(coarse_refresh, int) and coarse_refresh >= 1)):
            raise ValueError("coarse_refresh must be 'step', 'newton' or an int >= 1")
        self._coarse_refresh = coarse_refresh
        self._ew = (ew_gamma, ew_alpha)
        self._setup(mesh, np.array(rows, np.int32), np.array(tets, np.int32), up(np.concatenate(masses)),
                    up(np.concatenate(fexts)), up(np.concatenate(pins)), dt, tol, max_newton, precision, pcg_rtol,
                    pcg_max_iter, do_line_search, ls_threshold, profile, integrator)

    @classmethod
    def from_device(cls, mesh, inst_rows, inst_tets, mass, f_ext, pinned, dt=1.0 / 60.0, tol=1e-6, max_newton=20,
                    precision="mixed", pcg_rtol=-0.1, pcg_max_iter=4000, do_line_search=True, ls_threshold=None,
                    profile=False, integrator="be", graph=True, coarse_refresh="step", ew_gamma=0.9, ew_alpha=1.25):
        """A batch over an already concatenated device mesh: ``inst_rows`` / ``inst_tets`` (host
        int arrays, n_inst + 1) delimit the instances; mass (n), f_ext (3n) f64 and pinned (3n) u8
        are device tensors."""
        self = cls.__new__(cls)
        self.graph = graph
        if not (coarse_refresh in ("step", "newton") or (isinstance(coarse_refresh, int) and coarse_refresh >= 1)):
            raise ValueError("coarse_refresh must be 'step', 'newton' or an int >= 1")
        self._coarse_refresh = coarse_refresh
        self._ew = (ew_gamma, ew_alpha)
        self.n_inst = len(inst_rows) - 1
        if self.n_inst <= 0:
            raise ValueError("empty batch")
        self._setup(mesh, np.asarray(inst_rows, np.int32), np.asarray(inst_tets, np.int32), mass, f_ext, pinned,
                    dt, tol, max_newton, precision, pcg_rtol, pcg_max_iter, do_line_search, ls_threshold, profile,
                    integrator)
        return self

    def _setup(self, mesh, inst_rows_host, inst_tets_host, mass, f_ext, pinned, dt, tol, max_newton, precision,
               pcg_rtol, pcg_max_iter, do_line_search, ls_threshold, profile, integrator="be"):
        self.inst_rows_host = inst_rows_host
        self.inst_tets_host = inst_tets_host
        self.mesh = mesh
        m = self.mesh
        dev = m.device
        sizes = np.diff(self.inst_rows_host)
        up = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        self.inst_rows = up(self.inst_rows_host)
        self.inst_tets = up(self.inst_tets_host)
        self.vert_inst = up(np.repeat(np.arange(self.n_inst, dtype=np.int32), sizes))
        self.tet_inst = up(np.repeat(np.arange(self.n_inst, dtype=np.int32), np.diff(self.inst_tets_host)))
        self.order = up(np.argsort(-sizes, kind="stable").astype(np.int32))
        self.batch = BatchC(n_inst=self.n_inst, max_rows=int(sizes.max()), inst_rows=self.inst_rows.data_ptr(),
                            inst_tets=self.inst_tets.data_ptr(), vert_inst=self.vert_inst.data_ptr(),
                            tet_inst=self.tet_inst.data_ptr(), order=self.order.data_ptr())
        self.precision = PRECISIONS[precision]
        self.mass = mass
        self.f_ext = f_ext
        self.pinned = pinned
        self.u_prev = torch.zeros(3 * m.n, dtype=torch.float64, device=dev)
        self.u_curr = torch.zeros_like(self.u_prev)
        self.u_next = torch.zeros_like(self.u_prev)
        if integrator not in INTEGRATORS:
            raise ValueError(f"integrator must be one of {sorted(INTEGRATORS)}")
        self.integrator = integrator
        self.u_prev2 = torch.zeros_like(self.u_prev) if integrator == "bdf2" else None
        self.u_prev3 = torch.zeros_like(self.u_prev) if integrator == "bdf2" else None
        nbytes = _lib.load().skg_batch_workspace_size(ctypes.byref(m.c), ctypes.byref(self.batch), self.precision)
        if nbytes < 0:
            raise ValueError(_lib.last_error())
        self.workspace = torch.zeros(int(nbytes), dtype=torch.uint8, device=dev)
        self.params = BEParamsC(
            dt=dt, tol=tol, max_newton=max_newton, precision=self.precision, pcg_rtol=pcg_rtol,
            pcg_max_iter=pcg_max_iter, do_line_search=int(do_line_search), ls_alpha=0.01, ls_beta=0.5,
            ls_max_iter=100, pcg_mode=2,
            ls_threshold=(-1.0 if precision == "mixed" else 1e-12) if ls_threshold is None else ls_threshold,
            profile=int(profile), integrator=INTEGRATORS[integrator],
            coarse_refresh=int(getattr(self, "_coarse_refresh", "step") == "newton"),
            ew_gamma=self._ew[0], ew_alpha=self._ew[1])
        self._infos = (StepInfoC * self.n_inst)()
        self._coarse_age = None   # steps since the coarse inverses were built (integer refresh period)
        self._plans = {}          # device-loop graphs, one per rotation of the state buffers (and per
                                  # refresh decision with an integer refresh period)
        self._plan_key = None     # parameters and contact planes the plans were recorded with
        self._u_warm = None       # fixed buffer the warm start is copied into for the graphs
        init = getattr(self, "_contact_init", (None, True))
        self.set_contact_planes(*init)
        self.steps = 0

    def refresh_coarse(self):
        """With an integer refresh period: rebuild the per-instance coarse inverses at the next step
        (and count the period from there)."""
        self._coarse_age = None

    def set_contact_planes(self, planes, mass_weighted=True):
        """Contact springs against planes, each (k, p, n), for every instance."""
        self._planes, n = _lib.contact_planes(planes)
        self.params.n_planes = n
        self.params.contact_mass_weighted = int(bool(mass_weighted))
        self.params.planes = ctypes.cast(self._planes, ctypes.POINTER(_lib.ContactPlaneC))

    @property
    def n_tets(self):
        return self.mesh.t

    @property
    def n_verts(self):
        return self.mesh.n

    def step(self, u_warm=None, stream=None):
        """Advance every instance one step; returns (per-instance StepInfo list, total StepInfo).

        ``u_warm`` (3n, device FP64): optional Newton starting displacement, kept per
        instance only where its residual is below the residual at x_tilde.
        """
        bdf2 = self.integrator == "bdf2"
        st = BEStateC(u=self.u_next.data_ptr(), u_curr=self.u_curr.data_ptr(), u_prev=self.u_prev.data_ptr(),
                      mass=self.mass.data_ptr(), f_ext=self.f_ext.data_ptr(), pinned=self.pinned.data_ptr(),
                      u_warm=u_warm.data_ptr() if u_warm is not None else None,
                      u_prev2=self.u_prev2.data_ptr() if bdf2 else None,
                      u_prev3=self.u_prev3.data_ptr() if bdf2 else None, x_rest=self.mesh.X.data_ptr())
        total = StepInfoC()
        k = getattr(self, "_coarse_refresh", "step")
        if isinstance(k, int):
            rebuild = self._coarse_age is None or self._coarse_age + 1 >= k
            self.params.coarse_refresh = 0 if rebuild else -1
            self._coarse_age = 0 if rebuild else self._coarse_age + 1
        # a one-instance batch with coarse data inverts its coarse operator with a cooperative grid
        # launch, which stays on the host-driven path
        if self.graph and not self.params.profile and not (self.n_inst == 1 and bool(self.mesh.c.coarse)):
            if u_warm is not None:
                if self._u_warm is None:
                    self._u_warm = torch.empty_like(self.u_curr)
                self._u_warm.copy_(u_warm)
                st.u_warm = self._u_warm.data_ptr()
            plan = self._plan(st)
            check(_lib.load().skg_be_batch_plan_step(plan, self._infos, ctypes.byref(total), _stream_ptr(stream)))
        else:
            check(_lib.load().skg_be_step_batched(ctypes.byref(self.mesh.c), ctypes.byref(self.batch),
                                                  ctypes.byref(self.params), ctypes.byref(st),
                                                  ctypes.c_void_p(self.workspace.data_ptr()), self._infos,
                                                  ctypes.byref(total), _stream_ptr(stream)))
        if bdf2:
            self.u_prev3, self.u_prev2, self.u_prev, self.u_curr, self.u_next = (
                self.u_prev2, self.u_prev, self.u_curr, self.u_next, self.u_prev3)
        else:
            self.u_prev, self.u_curr, self.u_next = self.u_curr, self.u_next, self.u_prev
        self.steps += 1
        conv = lambda c: StepInfo(c.newton_iters, c.pcg_iters, c.ls_trials, c.status, c.residual0, c.residual,
                                  c.min_alpha, c.energy, c.launches, c.t_hessian_ms, c.t_assemble_ms, c.t_pcg_ms,
                                  c.t_gradient_ms, c.t_energy_ms, c.warm_used)
        return [conv(c) for c in self._infos], conv(total)

    def _params_key(self):
        """The parameters and contact planes the graphs depend on, less the per-step refresh decision
        (graphs for both decisions are kept)."""
        refresh = self.params.coarse_refresh
        self.params.coarse_refresh = 0
        raw = ctypes.string_at(ctypes.addressof(self.params), ctypes.sizeof(self.params))
        self.params.coarse_refresh = refresh
        planes = ctypes.string_at(ctypes.addressof(self._planes), ctypes.sizeof(self._planes)) if self._planes else b""
        return raw + planes

    def _plan(self, st):
        """The graph for this state binding and refresh decision (recorded on first use; all of them
        again after a change of the other parameters or of the contact planes)."""
        key = self._params_key()
        if key != self._plan_key:
            self.release_plans()
            self._plan_key = key
        bind = (st.u, st.u_curr, st.u_prev, st.u_prev2, st.u_prev3, st.u_warm, self.params.coarse_refresh)
        plan = self._plans.get(bind)
        if plan is None:
            h = ctypes.c_void_p()
            check(_lib.load().skg_be_batch_plan_create(ctypes.byref(self.mesh.c), ctypes.byref(self.batch),
                                                       ctypes.byref(self.params), ctypes.byref(st),
                                                       ctypes.c_void_p(self.workspace.data_ptr()), ctypes.byref(h)))
            plan = self._plans[bind] = h
        return plan

    def release_plans(self):
        for h in getattr(self, "_plans", {}).values():
            _lib.load().skg_be_batch_plan_destroy(h)
        self._plans = {}

    def __del__(self):
        try:
            self.release_plans()
        except Exception:
            pass

    def state(self):
        """Clones of the displacement levels (current first; four with BDF2)."""
        levels = [self.u_curr, self.u_prev] + ([self.u_prev2, self.u_prev3] if self.integrator == "bdf2" else [])
        return tuple(t.clone() for t in levels)

    def set_state(self, st):
        levels = [self.u_curr, self.u_prev] + ([self.u_prev2, self.u_prev3] if self.integrator == "bdf2" else [])
        for dst, src in zip(levels, st):
            dst.copy_(src)

    def displacement(self, inst=None) -> np.ndarray:
        u = self.u_curr.cpu().numpy()
        if inst is None:
            return u.copy()
        r0, r1 = self.inst_rows_host[inst], self.inst_rows_host[inst + 1]
        return u[3 * r0:3 * r1].copy()
