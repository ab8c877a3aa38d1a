"""Serving loop: beam-stepping requests batched on arrival, state resident in HBM.

Each request is one beam (seeded grid dims, Young's modulus, Poisson ratio and
gravity direction, pinned on its x = 0 face) asking for a number of
backward-Euler steps, each the ``backward_euler`` call of simkit
(``simkit/integrators/backward_euler.py:27-91``) with the stable neo-Hookean
closures.

The server keeps one device template per beam shape (nx, ny, nz): rest
positions, tets, inverse rest edge matrices and volumes (``skg_tet_setup``),
lumped masses, pins, and the block pattern with its assembly gather maps
(``device_pattern``: sorts on the device, the same maps the host builder
makes).  A cohort of requests is assembled on the device by concatenating
templates with index offsets, so admitting a request costs no host pattern
work, and is stepped by the batched solver until every request in it has
taken its steps; positions, velocities and patterns never leave the device.
Cohorts are admitted while free HBM (less a reserve) covers their estimated
footprint, and every live cohort advances one step per round (continuous
batching at cohort granularity).  Latency of a request = completion of its
last step - its arrival.
"""

from __future__ import annotations

import collections
import concurrent.futures
import os
import time
from dataclasses import dataclass, field
from types import SimpleNamespace

import numpy as np
import torch

from . import _lib
from .batched import BatchedBESolver
from .beams import _lame, beam_meshes
from .mesh import coarse_aggregates_inst, TetMesh, _ptr, _stream_ptr, device_pattern
from .solver import lumped_mass


@dataclass
class BeamRequest:
    rid: int
    dims: tuple
    ym: float
    pr: float
    gravity: np.ndarray
    steps: int
    t_arrival: float
    t_admit: float = -1.0
    t_done: float = -1.0


def request_stream(rate, duration, steps=10, seed=0, nx_range=(4, 16), ny_range=(4, 16), nz_range=(8, 48)):
    """Poisson arrivals at ``rate`` per second over ``duration`` seconds, each a seeded beam
    of the batched workload's distribution (nx, ny, nz uniform, E log-uniform [1e5, 1e7],
    nu uniform [0.30, 0.49], gravity 9.8 m/s^2 along a uniform direction)."""
    rng = np.random.default_rng(seed)
    n = rng.poisson(rate * duration)
    t = np.sort(rng.uniform(0.0, duration, size=n))
    nx = rng.integers(nx_range[0], nx_range[1] + 1, size=n)
    ny = rng.integers(ny_range[0], ny_range[1] + 1, size=n)
    nz = rng.integers(nz_range[0], nz_range[1] + 1, size=n)
    ym = np.exp(rng.uniform(np.log(1e5), np.log(1e7), size=n))
    pr = rng.uniform(0.30, 0.49, size=n)
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return [BeamRequest(i, (int(nx[i]), int(ny[i]), int(nz[i])), float(ym[i]), float(pr[i]), 9.8 * d[i], steps,
                        float(t[i])) for i in range(n)]


class ShapeTemplate:
    """Device data of one beam shape, as views into the storage of the chunk of shapes it was
    built with.  Index-valued arrays hold chunk-wide indices: ``vbase``, ``tbase`` and ``bbase``
    are the shape's first vertex, tet and block within its chunk."""

    __slots__ = ("dims", "n", "t", "nb", "X", "tets", "dinv", "vol", "mass", "pinned", "pattern", "vbase", "tbase",
                 "bbase", "coarse", "abase", "n_agg")


class TemplateCache:
    """Beam-shape templates on the device (cell 0.025 m, density 1000 kg/m^3, x = 0 face
    pinned).  Missing shapes are built together in chunks: the meshes by integer array
    arithmetic (``beam_meshes``), lumped masses on the host in tet order, inverse rest edge
    matrices and volumes by one ``skg_tet_setup`` launch, and the block pattern with its
    gather maps by one pair of device sorts (``device_pattern``)."""

    def __init__(self, device="cuda", chunk_tets=4_000_000, cell=0.025, rho=1000.0, coarse=True):
        self.coarse = coarse      # per-shape two-level aggregates (box 4) for the cluster PCG
        self.device = torch.device(device)
        self.chunk_tets = chunk_tets
        self.cell, self.rho = cell, rho
        self.shapes = {}
        self.build_s = 0.0
        self.bytes = 0

    def get(self, dims):
        dims = tuple(int(v) for v in dims)
        if dims not in self.shapes:
            self.ensure([dims])
        return self.shapes[dims]

    def ensure(self, dims_list):
        """Build every shape of ``dims_list`` not cached yet."""
        missing = sorted({tuple(int(v) for v in d) for d in dims_list} - set(self.shapes))
        if not missing:
            return
        t0 = time.perf_counter()
        chunks, chunk, tets = [], [], 0
        for d in missing:
            chunk.append(d)
            tets += 6 * d[0] * d[1] * d[2]
            if tets >= self.chunk_tets:
                chunks.append(chunk)
                chunk, tets = [], 0
        if chunk:
            chunks.append(chunk)
        if len(chunks) == 1:
            self._device_part(self._host_part(chunks[0]))
        else:
            # host meshes and masses in worker threads (numpy releases the interpreter lock),
            # device work in this thread as the chunks complete, in order
            workers = max(1, min(16, os.cpu_count() or 1, len(chunks)))
            with concurrent.futures.ThreadPoolExecutor(workers) as ex:
                for host in ex.map(self._host_part, chunks):
                    self._device_part(host)
        self.build_s += time.perf_counter() - t0

    def _host_part(self, dims):
        X, T, v_off, t_off = beam_meshes(dims, self.cell)
        mass = lumped_mass(X, T, self.rho)
        pin = np.zeros(3 * X.shape[0], np.uint8)
        for s, (nx, ny, nz) in enumerate(dims):       # vertices with i = 0 come first in each beam
            pin[3 * v_off[s]: 3 * (v_off[s] + (ny + 1) * (nz + 1))] = 1
        return dims, X, T.astype(np.int32), v_off, t_off, mass, pin

    def _device_part(self, host):
        dims, X, T, v_off, t_off, mass, pin = host
        lib = _lib.load()
        dev = self.device
        n, t = X.shape[0], T.shape[0]
        Xd = torch.from_numpy(X.reshape(-1)).to(dev)
        Td = torch.from_numpy(T).to(dev)
        dinv = torch.empty(9 * t, dtype=torch.float64, device=dev)
        vol = torch.empty(t, dtype=torch.float64, device=dev)
        _lib.check(lib.skg_tet_setup(_ptr(Xd), _ptr(Td), n, t, _ptr(dinv), _ptr(vol), _stream_ptr()))
        pattern = device_pattern(Td, n)
        massd = torch.from_numpy(mass).to(dev)
        pind = torch.from_numpy(pin).to(dev)
        b_off = pattern[0][torch.from_numpy(v_off).to(dev)].cpu().numpy().astype(np.int64)
        dinv2 = dinv.view(9, t)
        rowptr, col, diag, row, hc_ptr, hc_src, v2t_ptr, v2t = pattern
        self.bytes += sum(x.numel() * x.element_size() for x in (Xd, Td, dinv, vol, massd, pind, *pattern))
        cz = None
        if self.coarse:
            # per-shape aggregates over the chunk (chunk-wide aggregate and block indices, like the pattern)
            cd = coarse_aggregates_inst(X, pin.reshape(-1) == 0, rowptr.cpu().numpy(), col.cpu().numpy(), v_off,
                                        box=4)
            up = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
            cz = {"d": up(cd["mode"][:, :3]), "bits": up(cd["mode"][:, 3].view(np.int32)),
                  "colpack": up(cd["colpack"].view(np.int32)), "cb_ptr": up(cd["cb_ptr"]), "cb_slot": up(cd["cb_slot"]),
                  "cb_rc": up(cd["cb_rc"]), "inst_agg": cd["inst_agg"], "cb_ptr_h": cd["cb_ptr"],
                  "cb_first": np.searchsorted(cd["cb_rc"][0::2], cd["inst_agg"])}
            self.bytes += sum(v.numel() * v.element_size() for v in cz.values() if isinstance(v, torch.Tensor))
        for s, d in enumerate(dims):
            v0, v1, t0, t1, b0, b1 = (int(v_off[s]), int(v_off[s + 1]), int(t_off[s]), int(t_off[s + 1]),
                                      int(b_off[s]), int(b_off[s + 1]))
            tp = ShapeTemplate()
            tp.dims, tp.n, tp.t, tp.nb = d, v1 - v0, t1 - t0, b1 - b0
            tp.vbase, tp.tbase, tp.bbase = v0, t0, b0
            tp.X = Xd[3 * v0: 3 * v1]
            tp.tets = Td[t0:t1]
            tp.dinv = dinv2[:, t0:t1]
            tp.vol = vol[t0:t1]
            tp.mass = massd[v0:v1]
            tp.pinned = pind[3 * v0: 3 * v1]
            tp.pattern = (rowptr[v0: v1 + 1], col[b0:b1], diag[v0:v1], row[b0:b1], hc_ptr[b0: b1 + 1],
                          hc_src[16 * t0: 16 * t1], v2t_ptr[v0: v1 + 1], v2t[4 * t0: 4 * t1])
            tp.coarse = None
            if cz is not None:
                a0, a1 = int(cz["inst_agg"][s]), int(cz["inst_agg"][s + 1])
                c0, c1 = int(cz["cb_first"][s]), int(cz["cb_first"][s + 1])
                tp.abase, tp.n_agg = a0, a1 - a0
                tp.coarse = (cz["d"][v0:v1], cz["bits"][v0:v1], cz["colpack"][v0:v1], cz["cb_ptr"][c0: c1 + 1],
                             cz["cb_slot"][int(cz["cb_ptr_h"][c0]): int(cz["cb_ptr_h"][c1])], cz["cb_rc"][2 * c0: 2 * c1])
            self.shapes[d] = tp


def concat_patterns(parts, n_shift, t_shift, b_shift, nb_total, nt_total):
    """Pattern maps of a block-diagonal concatenation.  ``parts`` are per-instance
    (rowptr, col, diag, row, hc_ptr, hc_src, v2t_ptr, v2t) tuples whose values are shifted
    by the instance's vertex, tet and block shifts (new first index - index the part's
    values count from); nb_total, nt_total close the pointer arrays.  Equal to building the
    concatenated mesh's maps from scratch (every map is ordered by vertex, block or tet)."""
    dev = parts[0][0].device
    i32 = lambda v: torch.tensor([v], dtype=torch.int32, device=dev)
    rowptr = torch.cat([p[0][:-1] + b for p, b in zip(parts, b_shift)] + [i32(nb_total)])
    col = torch.cat([p[1] + v for p, v in zip(parts, n_shift)])
    diag = torch.cat([p[2] + b for p, b in zip(parts, b_shift)])
    row = torch.cat([p[3] + v for p, v in zip(parts, n_shift)])
    hc_ptr = torch.cat([p[4][:-1] + 16 * t for p, t in zip(parts, t_shift)] + [i32(16 * nt_total)])
    hc_src = torch.cat([p[5] + 16 * t for p, t in zip(parts, t_shift)])
    v2t_ptr = torch.cat([p[6][:-1] + 4 * t for p, t in zip(parts, t_shift)] + [i32(4 * nt_total)])
    v2t = torch.cat([p[7] + 4 * t for p, t in zip(parts, t_shift)])
    return rowptr, col, diag, row, hc_ptr, hc_src, v2t_ptr, v2t


def concat_coarse(tps, b_shift):
    """Per-instance two-level data of a cohort from the templates' pieces: aggregate indices
    shifted to the cohort's numbering, fine block slots by the pattern's block shifts, the coarse
    block pointers rebased; the packed column words hold instance-local aggregates and need none."""
    dev = tps[0].X.device
    na = np.array([tp.n_agg for tp in tps], np.int64)
    a_off = np.concatenate([[0], np.cumsum(na)])
    a_shift = [int(a_off[i] - tp.abase) for i, tp in enumerate(tps)]
    d = torch.cat([tp.coarse[0] for tp in tps])
    bits = torch.cat([tp.coarse[1] + a for tp, a in zip(tps, a_shift)])
    mode = torch.cat([d, bits.view(torch.float32)[:, None]], dim=1).contiguous()
    colpack = torch.cat([tp.coarse[2] for tp in tps])
    ns = np.array([tp.coarse[4].numel() for tp in tps], np.int64)
    s_off = np.concatenate([[0], np.cumsum(ns)])
    cb_ptr = torch.cat([tp.coarse[3][:-1] - tp.coarse[3][0] + int(o) for tp, o in zip(tps, s_off[:-1])]
                       + [torch.tensor([int(s_off[-1])], dtype=torch.int32, device=dev)])
    cb_slot = torch.cat([tp.coarse[4] + b for tp, b in zip(tps, b_shift)])
    cb_rc = torch.cat([tp.coarse[5] + a for tp, a in zip(tps, a_shift)])
    nps = ((6 * na + 31) // 32) * 32
    up = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a).astype(dt)).to(dev)
    return {"mode": mode, "colpack": colpack, "cb_ptr": cb_ptr.to(torch.int32), "cb_slot": cb_slot, "cb_rc": cb_rc,
            "inst_agg": up(a_off, np.int32), "agg_inst": up(np.repeat(np.arange(len(tps)), na), np.int32),
            "inst_moff": up(np.concatenate([[0], np.cumsum(nps * nps)]), np.int64)}


def build_cohort(cache, reqs, **solver_kw):
    """A BatchedBESolver over the requests' beams, assembled on the device from templates."""
    cache.ensure([r.dims for r in reqs])
    tps = [cache.get(r.dims) for r in reqs]
    ns = np.array([tp.n for tp in tps], np.int64)
    ts = np.array([tp.t for tp in tps], np.int64)
    bs = np.array([tp.nb for tp in tps], np.int64)
    n_off = np.concatenate([[0], np.cumsum(ns)])
    t_off = np.concatenate([[0], np.cumsum(ts)])
    b_off = np.concatenate([[0], np.cumsum(bs)])
    if 16 * t_off[-1] >= 2 ** 31:
        raise ValueError("cohort too large for int32 gather maps")
    dev = tps[0].X.device
    n_shift = [int(n_off[i] - tp.vbase) for i, tp in enumerate(tps)]
    t_shift = [int(t_off[i] - tp.tbase) for i, tp in enumerate(tps)]
    b_shift = [int(b_off[i] - tp.bbase) for i, tp in enumerate(tps)]
    X = torch.cat([tp.X for tp in tps])
    tets = torch.cat([tp.tets + v for tp, v in zip(tps, n_shift)])
    # inverse rest edge matrices are stored component-major (entry (i, j) of tet e at (3i + j) t + e)
    dinv = torch.cat([tp.dinv for tp in tps], dim=1).reshape(-1).contiguous()
    vol = torch.cat([tp.vol for tp in tps])
    mu_i, lam_i = _lame(np.array([r.ym for r in reqs]), np.array([r.pr for r in reqs]))
    tcount = torch.from_numpy(ts).to(dev)
    mu = torch.repeat_interleave(torch.from_numpy(mu_i).to(dev), tcount)
    lam = torch.repeat_interleave(torch.from_numpy(lam_i).to(dev), tcount)
    pattern = concat_patterns([tp.pattern for tp in tps], n_shift, t_shift, b_shift, int(b_off[-1]), int(t_off[-1]))
    mesh = TetMesh.from_device(X, tets, dinv, vol, mu, lam, pattern)
    if all(tp.coarse is not None for tp in tps):
        mesh.set_coarse_device(concat_coarse(tps, b_shift))
    mass = torch.cat([tp.mass for tp in tps])
    grav = torch.from_numpy(np.stack([r.gravity for r in reqs])).to(dev)
    f_ext = (mass[:, None] * torch.repeat_interleave(grav, torch.from_numpy(ns).to(dev), dim=0)).reshape(-1)
    pinned = torch.cat([tp.pinned for tp in tps])
    solver = BatchedBESolver.from_device(mesh, n_off.astype(np.int32), t_off.astype(np.int32), mass,
                                         f_ext.contiguous(), pinned, **solver_kw)
    specs = [SimpleNamespace(ym=np.array([r.ym]), pr=np.array([r.pr]), dims=r.dims) for r in reqs]
    return solver, specs


@dataclass
class Cohort:
    solver: BatchedBESolver
    reqs: list
    fb: object = None
    steps_done: int = 0
    tets: int = 0


@dataclass
class ServeStats:
    duration_s: float = 0.0
    elapsed_s: float = 0.0
    arrived: int = 0
    admitted: int = 0
    completed: int = 0
    backlog: int = 0
    instance_steps: int = 0
    rounds: int = 0
    cohorts: int = 0
    latency_ms: list = field(default_factory=list)
    wait_ms: list = field(default_factory=list)
    failed_steps: int = 0
    template_build_s: float = 0.0
    cohort_build_s: float = 0.0
    peak_live: int = 0
    warm_kept: list = field(default_factory=list)

    def summary(self):
        lat = np.array(self.latency_ms) if self.latency_ms else np.array([np.nan])
        wait = np.array(self.wait_ms) if self.wait_ms else np.array([np.nan])
        return {
            "duration_s": self.duration_s, "elapsed_s": self.elapsed_s, "arrived": self.arrived,
            "admitted": self.admitted, "completed": self.completed, "backlog_at_end": self.backlog,
            "instance_steps_per_s": self.instance_steps / max(self.elapsed_s, 1e-9),
            "completed_requests_per_s": self.completed / max(self.elapsed_s, 1e-9),
            "latency_ms_p50": float(np.percentile(lat, 50)), "latency_ms_p99": float(np.percentile(lat, 99)),
            "latency_ms_mean": float(np.mean(lat)), "queue_wait_ms_p50": float(np.percentile(wait, 50)),
            "queue_wait_ms_p99": float(np.percentile(wait, 99)), "rounds": self.rounds, "cohorts": self.cohorts,
            "peak_live_requests": self.peak_live, "failed_steps": self.failed_steps,
            "template_build_s": self.template_build_s, "cohort_build_s": self.cohort_build_s,
            "warm_start_kept_fraction": float(np.mean(self.warm_kept)) if self.warm_kept else None,
        }


class BeamServer:
    """Continuous-batching server for beam-stepping requests on one GPU.

    max_cohort: requests per cohort; max_live: requests in flight; hbm_reserve_gb: HBM
    left free; net: a trained ``WarmStartMLP`` (the learned warm start with its
    residual-judged fallback) or None for plain Newton starts; coarse: two-level PCG with
    per-shape aggregates (built with the templates)."""

    def __init__(self, max_cohort=512, max_live=2048, hbm_reserve_gb=16.0, net=None, device="cuda",
                 coarse=True, **solver_kw):
        self.cache = TemplateCache(device, coarse=coarse)
        self.prewarm_s = 0.0
        self.max_cohort = max_cohort
        self.max_live = max_live
        self.reserve = hbm_reserve_gb * 2 ** 30
        self.net = net
        self.solver_kw = solver_kw
        self.bytes_per_tet = 4096.0  # recalibrated from every cohort built

    def prewarm(self, dims_list):
        """Build the templates of a shape catalog ahead of traffic."""
        t0 = time.perf_counter()
        self.cache.ensure(dims_list)
        torch.cuda.synchronize()
        self.prewarm_s += time.perf_counter() - t0

    def _admit(self, pending, live_reqs):
        free = torch.cuda.mem_get_info()[0] - self.reserve
        take = []
        while pending and len(take) < self.max_cohort and live_reqs + len(take) < self.max_live:
            r = pending[0]
            nx, ny, nz = r.dims
            need = self.bytes_per_tet * 6 * nx * ny * nz
            if need > free:
                break
            free -= need
            take.append(pending.popleft())
        return take

    def _step(self, c, st):
        if self.net is not None:
            from .warmstart import warm_step
            infos, total = warm_step(c.solver, c.fb, self.net)
            st.warm_kept.append(sum(i.warm_used for i in infos) / len(infos))
        else:
            infos, total = c.solver.step()
        if total.status != 0:
            st.failed_steps += sum(1 for i in infos if i.status != 0)
        c.steps_done += 1

    def run(self, requests, duration, serve_backlog=False):
        """Serve ``requests`` (sorted by arrival) arriving over ``duration`` seconds.  Admission
        stops at ``duration`` (the backlog is reported) unless ``serve_backlog``, and the live
        cohorts are drained.  Returns ServeStats."""
        st = ServeStats(duration_s=duration)
        pending = collections.deque()
        live = []
        nxt = 0
        t0 = time.perf_counter()
        while True:
            now = time.perf_counter() - t0
            while nxt < len(requests) and requests[nxt].t_arrival <= min(now, duration):
                pending.append(requests[nxt])
                nxt += 1
            live_reqs = sum(len(c.reqs) for c in live)
            admitting = now < duration or (serve_backlog and nxt >= len(requests))
            if admitting and pending and live_reqs < self.max_live:
                take = self._admit(pending, live_reqs)
                if take:
                    tb = time.perf_counter()
                    t_tpl = self.cache.build_s
                    m0 = torch.cuda.memory_allocated()
                    solver, specs = build_cohort(self.cache, take, **self.solver_kw)
                    c = Cohort(solver, take, tets=solver.n_tets)
                    if self.net is not None:
                        from .warmstart import FeatureBuilder
                        c.fb = FeatureBuilder(solver, specs)
                    torch.cuda.synchronize()
                    used = torch.cuda.memory_allocated() - m0
                    self.bytes_per_tet = max(1024.0, used / max(c.tets, 1))
                    st.cohort_build_s += time.perf_counter() - tb - (self.cache.build_s - t_tpl)
                    st.template_build_s = self.cache.build_s
                    ta = time.perf_counter() - t0
                    for r in take:
                        r.t_admit = ta
                    live.append(c)
                    st.cohorts += 1
                    st.admitted += len(take)
                    st.peak_live = max(st.peak_live, live_reqs + len(take))
            if not live:
                if (now >= duration and not (serve_backlog and pending)) or (nxt >= len(requests) and not pending):
                    break
                wait = (requests[nxt].t_arrival - now) if nxt < len(requests) else 0.001
                time.sleep(min(max(wait, 0.0), 0.01))
                continue
            for c in live:
                self._step(c, st)
                st.instance_steps += len(c.reqs)
            st.rounds += 1
            finished = [c for c in live if c.steps_done >= c.reqs[0].steps]
            if finished:
                torch.cuda.synchronize()
                td = time.perf_counter() - t0
                for c in finished:
                    for r in c.reqs:
                        r.t_done = td
                        st.latency_ms.append(1e3 * (td - r.t_arrival))
                        st.wait_ms.append(1e3 * (r.t_admit - r.t_arrival))
                    st.completed += len(c.reqs)
                live = [c for c in live if c.steps_done < c.reqs[0].steps]
        st.elapsed_s = time.perf_counter() - t0
        st.arrived = nxt
        st.backlog = len(pending)
        return st
