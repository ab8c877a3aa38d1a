#!/usr/bin/env python
"""Benchmark of the backward-Euler stable neo-Hookean path on one GB300.

Workload: the 32 x 32 x 128-cube beam (786,432 tets, 140,481 vertices, rest
shape jittered by U(-0.1, 0.1) cells, Young's modulus log-uniform [1e5, 1e7]
per tet, nu = 0.45, rho = 1000, gravity -y, x = 0 face pinned), dt = 1/60,
Newton to 1e-6 relative residual (<= 20 iterations), FP32 element Hessians
and SpMV with FP64 gradient, residual, dots and energy sums.

A step is one Newton-converged backward-Euler step.  `value` is steps/s with
the state resident in HBM; `e2e` is the same metric through the host-buffer
entry point (positions copied host->device and back inside the timed region).
Every input of the timed region (matrix 81 MB, per-tet Hessian records
252 MB) is larger than the 129 MB L2, so no L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Newton-converged steps/s & tet-Hessians/s, plain vs batched+learned @1e-6 resid"
WORKLOAD = "beam 32x32x128 cubes, 786,432 tets, jittered, E log-uniform [1e5,1e7], 1 instance, plain Newton"
SMALL_WORKLOAD = "beam 8x8x32 cubes, 12,288 tets, E 1e6, nu 0.45 (quick check)"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ CPU baseline
def host_cpu():
    """CPU model (lscpu), logical cores and the BLAS/OpenMP thread setting of this process."""
    model = None
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.split(":")[0].strip() in ("Model name", "Model"):
                model = ln.split(":", 1)[1].strip()
                if ln.startswith("Model name"):
                    break
    except Exception:
        pass
    return {"model": model, "logical_cores": os.cpu_count(),
            "omp_num_threads": os.environ.get("OMP_NUM_THREADS", "default")}


def slab_of(spec, layers):
    """The first ``layers`` cube layers (along x, from the pinned face) of a beam: a complete,
    smaller beam with the same jitter, materials and pins (vertices and tets are numbered x-major)."""
    nx, ny, nz = spec.dims
    nv = (layers + 1) * (ny + 1) * (nz + 1)
    nt = 6 * layers * ny * nz
    return nv, nt


class CpuReferenceSteps:
    """simkit's FP64 numpy/scipy step (the oracle restatement: its energies, Hessians with the
    eigenvalue floor, block_diag / J^T H J assembly, scipy spsolve, Armijo line search, Newton to
    the 1e-6 relative residual) run for real on a slab of the workload beam, one backward-Euler
    step per call, on a rollout from rest that restarts every ``restart`` steps (the stiff slab
    comes to rest within a few steps, after which the relative residual measures FP64 noise; the
    headline beam is still swinging).  Every call is a measured full step (the direct solve
    included).  The whole-mesh figure scales the measured step time by tet count: the sparse direct
    solve grows faster than linearly with the mesh (a slab twice as long takes 3x as long per
    step), so the linear figure is an upper bound on the reference's steps/s."""

    def __init__(self, spec, layers=2, restart=4):
        from oracle import rollout
        nv, nt = slab_of(spec, layers)
        self.layers, self.nt, self.full_tets = layers, nt, spec.n_tets
        self.restart = restart
        self.r = rollout.BeamRollout(spec.X[:nv], spec.T[:nt], spec.mu[:nt], spec.lam[:nt], spec.rho,
                                     spec.gravity, spec.pinned, 1.0 / 60.0)
        self.times, self.iters = [], []
        self.not_converged = 0

    def step(self):
        if len(self.times) % self.restart == 0:
            self.x_prev = self.r.x_rest.copy()
            self.x_curr = self.r.x_rest.copy()
        t0 = time.perf_counter()
        x_next, info = self.r.step(self.x_curr, self.x_prev)
        dt = time.perf_counter() - t0
        self.not_converged += int(not info.converged)
        self.x_prev, self.x_curr = self.x_curr, x_next
        self.times.append(dt)
        self.iters.append(info.iters)
        return dt

    def summary(self, skip=0):
        t = np.array(self.times[skip:])
        ms = 1e3 * float(t.mean())
        per_full_step_s = float(t.mean()) * self.full_tets / self.nt
        return {
            "measured_ms_per_step": ms,
            "measured_steps_per_s": 1e3 / ms,
            "measured_tet_hessians_per_s": self.nt * float(np.mean(self.iters[skip:])) / float(t.mean()),
            "newton_iters_per_step": float(np.mean(self.iters[skip:])),
            "steps_not_converged": self.not_converged,
            "extrapolated_steps_per_s": 1.0 / per_full_step_s,
            "sample": (f"{len(t)} measured backward-Euler steps (Newton to 1e-6 with scipy spsolve and Armijo "
                       f"search, FP64) of the first {self.layers} cube layers of the workload beam "
                       f"({self.nt} tets, same jitter, materials and pinned face), rollouts from rest of "
                       f"{self.restart} steps; steps/s for the {self.full_tets}-tet mesh = measured step time x "
                       f"{self.full_tets / self.nt:.0f} (tet ratio): an upper bound, the direct solve "
                       "grows faster than linearly"),
        }


# --------------------------------------------------------------- helpers
def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Ranks:
    """Replica bookkeeping under torchrun: every rank steps its own independent meshes (no
    data-path collective); the process group carries only the barriers around the timed region
    and the max-over-ranks time.  Backend "nccl" on the GPUs, "gloo" for ranks on CPU."""

    def __init__(self, backend="nccl"):
        self.ws, self.rank, self.local = dist_setup()
        self.dist = None
        self.device = "cuda" if backend == "nccl" else "cpu"
        if self.ws > 1:
            import torch.distributed as dist
            dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def whole_job_rate(self, units_per_rank: float, seconds_max: float) -> float:
        """Units all ranks processed / the slowest rank's time."""
        return units_per_rank * self.ws / seconds_max

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def replica_seed(rank: int) -> int:
    """Seed of a rank's replica: rank 0 runs the published workload (seed 0), rank r its own
    seeded draw of the same distribution."""
    return int(rank)


def _refresh_arg(v):
    if v in ("step", "newton"):
        return v
    k = int(v)
    if k < 1:
        raise ValueError("refresh interval must be >= 1")
    return k


def algorithmic_bytes(spec, nb, n_coarse=0):
    n, t = spec.n_verts, spec.n_tets
    return {
        # one tet-Hessian (evaluated, projected, assembled): tets 16 + shape operator 36
        # + material 12 + positions 12 n/t + block values written once 4 * 9 nb / t
        "tet_hessian": 16 + 36 + 12 + 12.0 * n / t + 36.0 * nb / t,
        # one PCG iteration: block values + column indices + row pointers,
        # SpMV p read / q write, update x r p q read + x r z write, Jacobi blocks,
        # direction z p read + p write (12 useful bytes per vertex vector); with the
        # two-level preconditioner also the dense coarse inverse (4 n_c^2), the column's
        # coarse word per block (8 nb), the per-vertex coarse data read by the restriction
        # (16 n) and the coarse vectors (P^T r as 8-byte integers written and read, e)
        "pcg_iter": 40.0 * nb + 4.0 * (n + 1) + 24.0 * n + 84.0 * n + 36.0 * n + 36.0 * n
                    + (4.0 * n_coarse * n_coarse + 8.0 * nb + 16.0 * n + 20.0 * n_coarse if n_coarse else 0.0),
    }


def parity_report(spec, solver_kw, steps_fp64=30):
    """Errors of the timed configuration on the workload beam (seed 0), outside the timed region:
    (1) the first two steps from rest against simkit's own steps stored in
    tests/golden/rollout_beam_32x32x128_first_steps.npz (simkit's spsolve replaced there by a 1e-10
    PCG; sampled vertices); (2) ``steps_fp64`` steps against the package's FP64 mode (FP64 kernels,
    PCG forcing 1e-3).  Positions relative to the largest rest coordinate, displacements relative
    to the largest displacement."""
    from simkit_gb300.solver import BESolver
    out = {}
    scale = float(np.abs(spec.X).max())
    path = os.path.join(ROOT, "tests", "golden", "rollout_beam_32x32x128_first_steps.npz")
    if os.path.exists(path):
        d = np.load(path)
        s = BESolver.from_spec(spec, **solver_kw)
        pos = disp = 0.0
        for k, step in enumerate(d["steps"]):
            while s.steps < int(step):
                if not s.step().converged:
                    raise SystemExit("parity step did not converge")
            u = s.displacement().reshape(-1, 3)[d["sample"]]
            pos = max(pos, float(np.abs(u - d["u"][k]).max()) / scale)
            disp = max(disp, float(np.abs(u - d["u"][k]).max() / np.abs(d["u"][k]).max()))
        out["vs_simkit"] = {"steps": int(d["steps"].max()), "positions_rel": pos, "displacement_rel": disp,
                            "vertices": int(d["sample"].size),
                            "reference": "simkit's energies, Hessians, line search and Newton; " + str(d["solve"])}
        del s
    a = BESolver.from_spec(spec, **solver_kw)
    kw64 = dict(solver_kw, precision="fp64", pcg_rtol=1e-3)
    b = BESolver.from_spec(spec, **kw64)
    pos = disp = 0.0
    for _ in range(steps_fp64):
        if not (a.step().converged and b.step().converged):
            raise SystemExit("parity step did not converge")
        ua, ub = a.displacement(), b.displacement()
        pos = max(pos, float(np.abs(ua - ub).max()) / scale)
        disp = max(disp, float(np.abs(ua - ub).max() / np.abs(ub).max()))
    out["vs_fp64_mode"] = {"steps": steps_fp64, "positions_rel": pos, "displacement_rel": disp}
    return out


def dropin_summary(steps=10, warmup=2, cpu_steps=2):
    """simkit's own call on the device fast path: ``backward_euler`` handed an ElasticPotential's
    closures and a lumped M (FP64, the linear solves to 1e-12, simkit's stop rule ||alpha dx|| < 1e-6
    with up to 20 Newton iterations, the step's positions in and out as host arrays) on the
    12,288-tet 8 x 8 x 32 beam (E 1e6, nu 0.45, gravity, no pins: simkit's integrator takes none),
    timed on the host clock over ``steps`` steps after ``warmup``."""
    import scipy.sparse as sps
    import torch
    from simkit_gb300 import api
    from simkit_gb300.beams import make_beam
    from simkit_gb300.solver import lumped_mass
    spec = make_beam(8, 8, 32, ym=1e6, pr=0.45)
    m = lumped_mass(spec.X, spec.T, spec.rho)
    M = sps.diags(np.repeat(m, 3)).tocsc()
    f = (m[:, None] * spec.gravity[None, :]).reshape(-1, 1)
    pot = api.ElasticPotential(spec.X, spec.T, spec.mu, spec.lam, f_ext=f)
    h = 1.0 / 60.0
    x_prev = spec.X.reshape(-1, 1).copy()
    x_curr = x_prev.copy()
    t0 = None
    for k in range(warmup + steps):
        if k == warmup:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
        x_next = api.backward_euler(x_curr, x_prev, pot.energy, pot.gradient, pot.hessian, M, h,
                                    tolerance=1e-6, max_iter=20)
        x_prev, x_curr = x_curr, x_next
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    out = {"workload": "simkit.backward_euler(x_curr, x_prev, pot.energy, pot.gradient, pot.hessian, M, h, "
                       "tolerance=1e-6, max_iter=20) on the 8 x 8 x 32 beam (12,288 tets), ElasticPotential "
                       "closures, lumped M, FP64, host arrays in and out",
           "steps": steps, "steps_per_s": steps / dt, "ms_per_step": 1e3 * dt / steps,
           "stepper": "device fast path (one BESolver per (h, M))" if len(pot._steppers) == 1 else "closure path"}
    if cpu_steps > 0:
        # the same call on the oracle (simkit's backward_euler / newton_solver with spsolve), same start
        from oracle import fem, snh as osnh, solvers as osol
        J, vol = fem.deformation_jacobian(spec.X, spec.T), fem.tet_volumes(spec.X, spec.T)
        Eo = lambda x: osnh.energy_x(x, J, spec.mu, spec.lam, vol) - float((f.T @ x).item())
        Go = lambda x: osnh.gradient_x(x, J, spec.mu, spec.lam, vol) - f
        Ho = lambda x: osnh.hessian_x(x, J, spec.mu, spec.lam, vol)
        x_prev = spec.X.reshape(-1, 1).copy()
        x_curr = x_prev.copy()
        t0 = time.perf_counter()
        for _ in range(cpu_steps):
            x_next = osol.backward_euler(x_curr, x_prev, Eo, Go, Ho, M, h, tolerance=1e-6, max_iter=20)
            x_prev, x_curr = x_curr, x_next
        cdt = time.perf_counter() - t0
        out["oracle_steps_per_s"] = cpu_steps / cdt
        out["oracle_sample"] = (f"the oracle's backward_euler (simkit's algorithm, spsolve) on the host cores, the "
                                f"first {cpu_steps} steps from rest, same call")
    return out


def batched_summary(instances=128, steps=4, warmup=3, plain_sample=4, train_steps=12, seed=0, coarse_refresh=8):
    """Reduced 512-beam workload for the headline line: ``instances`` beams of the same seeded
    distribution (nx, ny in 4..16, nz in 8..48, own E, nu and gravity direction) stepped together
    (the device-resident Newton loop: one graph launch per step), against a sample of the same beams
    stepped one at a time by the single-instance solver (two-level cluster PCG and the one-level
    block-Jacobi form first specified), and the batch with the learned warm start (a network
    trained here on frames of a separately seeded batch).  Times by CUDA events; not part of the
    headline's timed region."""
    import torch
    from simkit_gb300 import warmstart as wsm
    from simkit_gb300.autotune import tune_pcg_variant
    from simkit_gb300.batched import BatchedBESolver
    from simkit_gb300.beams import beam_batch
    from simkit_gb300.solver import BESolver
    stream = torch.cuda.current_stream()

    def timed(fn, k):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = [fn() for _ in range(k)]
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out

    specs = beam_batch(instances, seed=seed)
    b = BatchedBESolver(specs, coarse_refresh=coarse_refresh)
    for _ in range(warmup):
        b.step()
    b.refresh_coarse()     # every timed window starts with fresh coarse inverses
    ms, outs = timed(b.step, steps)
    if any(t.status != 0 for _, t in outs):
        raise SystemExit("batched summary: a step failed")
    batched = instances * steps / (ms / 1000.0)
    newton = sum(t.newton_iters for _, t in outs) / (instances * steps)
    pick = np.random.default_rng(1).choice(instances, size=plain_sample, replace=False)

    def plain(coarse):
        per = []
        for i in pick:
            s1 = BESolver.from_spec(specs[i], coarse=coarse, coarse_refresh=coarse_refresh)
            for _ in range(warmup):
                s1.step()
            tune_pcg_variant(s1)
            s1.refresh_coarse()
            m1, _ = timed(s1.step, steps)
            per.append(m1 / steps)
        return 1000.0 / float(np.mean(per))
    plain_2l, plain_bj = plain("auto"), plain(None)
    # learned warm start: trained on a separate seeded batch of the same distribution
    tspecs = beam_batch(instances, seed=100 + seed)
    tb = BatchedBESolver(tspecs)
    frames, _ = wsm.generate_frames(tb, tspecs, train_steps)
    net = wsm.WarmStartMLP(seed=0, lr=1e-3)
    wsm.train(net, tb, frames, epochs=2, batch_frames=64)
    del frames, tb
    bl = BatchedBESolver(specs, coarse_refresh=coarse_refresh)
    fb = wsm.FeatureBuilder(bl, specs)
    for _ in range(warmup):
        ut = fb.u_tilde()
        bl.step()
        fb.record_correction(ut)
    bl.refresh_coarse()
    ml, louts = timed(lambda: wsm.warm_step(bl, fb, net), steps)
    learned = instances * steps / (ml / 1000.0)
    return {
        "workload": f"{instances} beams of the 512-beam distribution, {steps} timed steps after {warmup}",
        "batched_instance_steps_per_s": batched, "newton_iters_per_instance_step": newton,
        "plain_single_instance": plain_2l, "plain_single_instance_block_jacobi": plain_bj,
        "plain_sample": f"{plain_sample} of the beams stepped alone, {steps} steps each after {warmup}",
        "batched_over_plain": batched / plain_2l, "batched_over_plain_block_jacobi": batched / plain_bj,
        "learned_instance_steps_per_s": learned,
        "learned_newton_iters_per_instance_step": sum(t.newton_iters for _, t in louts) / (instances * steps),
        "learned_kept_fraction": float(np.mean([sum(i.warm_used for i in inf) / len(inf) for inf, _ in louts])),
        "learned_over_plain_block_jacobi": learned / plain_bj,
        "learned_training": f"{instances} beams x {train_steps} steps of frames, 2 epochs, Adam lr 1e-3",
    }


def run_reference(args):
    """The reference's CPU path (the oracle restatement of simkit's algorithm) on the machine's host:
    each bench step is one measured backward-Euler step of a slab of the workload beam, the direct
    solve included (CpuReferenceSteps).  ms_per_step is that measured time; value is the whole-mesh
    steps/s extrapolated from it (labelled, an upper bound)."""
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    from simkit_gb300.beams import beam_large_jittered, beam_small_steady
    if args.small:
        # the 12,288-tet beam is small enough to time whole: a plain rollout from rest, nothing scaled
        spec = beam_small_steady()
        ref = CpuReferenceSteps(spec, layers=spec.dims[0], restart=10 ** 9)
    else:
        spec = beam_large_jittered()
        ref = CpuReferenceSteps(spec, layers=args.ref_layers)
    t0 = time.perf_counter()
    for _ in range(args.warmup + args.steps):
        ref.step()
    wall = time.perf_counter() - t0
    sm = ref.summary(skip=args.warmup)
    v = sm["extrapolated_steps_per_s"]
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sm["measured_ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": SMALL_WORKLOAD if args.small else WORKLOAD, "precision": "fp64 numpy/scipy",
                   "l2": "inputs larger than L2"},
        "value_kind": ("measured: the whole beam, a rollout from rest" if args.small else
                       "extrapolated from the measured slab steps (linear in tets, an upper bound)"),
        "ms_per_step_kind": "measured: one full backward-Euler step of the slab sample",
        "measured": sm, "wall_s": wall, "host": host_cpu(),
        "tet_hessians_per_s": sm["measured_tet_hessians_per_s"],
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": 1, "kind": "port", "sample": sm["sample"],
                         "threads": "numpy/scipy as simkit runs them: element math and SuperLU single-threaded"},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def train_warm_start(args):
    """The warm-start MLP trained on frames the plain batched solver generates on a separate
    seeded batch of beams (tensor-core forward/backward, Adam).  Returns (net, info)."""
    import torch
    from simkit_gb300 import warmstart as ws
    from simkit_gb300.batched import BatchedBESolver
    from simkit_gb300.beams import beam_batch
    t0 = time.perf_counter()
    train_specs = beam_batch(args.instances, seed=100)
    coarse = None if args.coarse == "none" else (args.coarse if args.coarse == "auto" else int(args.coarse))
    tb = BatchedBESolver(train_specs, precision=args.precision, pcg_rtol=args.pcg_rtol, coarse=coarse)
    frames, _ = ws.generate_frames(tb, train_specs, args.train_steps)
    t_gen = time.perf_counter() - t0
    net = ws.WarmStartMLP(seed=0, lr=1e-3)
    t0 = time.perf_counter()
    losses = ws.train(net, tb, frames, epochs=args.epochs, batch_frames=64)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del frames, tb
    per_epoch = max(1, len(losses) // max(args.epochs, 1))
    return net, {"frames": args.instances * args.train_steps, "generate_s": t_gen, "train_s": t_train,
                 "adam_steps": len(losses), "loss_first_epoch": float(np.mean(losses[:per_epoch])),
                 "loss_last_epoch": float(np.mean(losses[-per_epoch:]))}


def run_serving(args):
    """A Poisson stream of beam requests (the 512-beam workload's distribution, 10 steps each)
    served by continuous batching at cohort granularity for ``--duration`` seconds; latency per
    request = completion of its 10th step - arrival.  Metric unit: instance-steps/s."""
    import torch
    from simkit_gb300.serving import BeamServer, request_stream
    if dist_setup()[1] != 0:
        # one server on one GPU: under torchrun the other ranks have no work
        return 0
    torch.cuda.set_device(0)
    net, learned = (None, None)
    if args.learned:
        net, learned = train_warm_start(args)
    reqs = request_stream(args.rate, args.duration, steps=10, seed=0)
    srv = BeamServer(max_cohort=args.max_cohort, max_live=args.max_live, net=net, precision=args.precision,
                     pcg_rtol=args.pcg_rtol, coarse=args.coarse != "none", graph=not args.no_graph,
                     coarse_refresh=args.batched_coarse_refresh)
    # the shape catalog (every nx, ny in 4..16, nz in 8..48) is built before traffic starts
    catalog = [(a, b, c) for a in range(4, 17) for b in range(4, 17) for c in range(8, 49)]
    srv.prewarm(catalog)
    clocks = ClockSampler(0)
    clocks.start()
    st = srv.run(reqs, args.duration)
    clock_info = clocks.stop()
    sm = st.summary()
    line = {
        "metric": METRIC, "value": sm["instance_steps_per_s"], "unit": "instance-steps/s", "n_gpus": 1,
        "steps": sm["rounds"], "warmup": 0, "ms_per_step": 1e3 * st.elapsed_s / max(sm["rounds"], 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": f"serving: Poisson {args.rate:g} requests/s for {args.duration:g} s, each a beam "
                               "(nx, ny in 4..16, nz in 8..48) asking for 10 backward-Euler steps"
                               + (", learned warm start" if args.learned else ", plain Newton"),
                   "rate": args.rate, "duration_s": args.duration, "max_cohort": args.max_cohort,
                   "max_live": args.max_live, "precision": args.precision,
                   "newton_loop": "host" if args.no_graph else "device (CUDA graph)"},
        "serving": sm, "learned": learned, "clocks": clock_info,
        "catalog": {"shapes": len(srv.cache.shapes), "build_s": srv.prewarm_s,
                    "device_bytes": srv.cache.bytes},
    }
    print(json.dumps(line))
    return 0


def run_batched(args):
    """512 seeded beams (nx, ny in {4..16}, nz in {8..48}, own E, nu, gravity direction),
    all stepped together; compared with stepping a sample of the same beams one at a
    time through the single-instance solver.  Metric unit: instance-steps/s."""
    import torch
    from simkit_gb300.batched import BatchedBESolver
    from simkit_gb300.beams import beam_batch
    from simkit_gb300.solver import BESolver
    from simkit_gb300.sharding import gather_to_rank0, shard
    n_ranks, rank, local = dist_setup()
    torch.cuda.set_device(local)
    ranks = Ranks("nccl")
    # one batch of args.instances beams split across the ranks by LPT on tet count (instances are
    # independent: no exchange in the solve); per-instance results are gathered on rank 0 at the end
    specs_all = beam_batch(args.instances, seed=0)
    shard_idx, specs = shard(specs_all, rank, n_ranks)
    # the same preconditioner on both sides of the comparison: two-level (per-instance
    # aggregates) unless --coarse none
    coarse = None if args.coarse == "none" else (args.coarse if args.coarse == "auto" else int(args.coarse))
    b = BatchedBESolver(specs, precision=args.precision, pcg_rtol=args.pcg_rtol, coarse=coarse,
                        coarse_refresh=args.batched_coarse_refresh, graph=not args.no_graph,
                        ew_alpha=args.batched_ew_alpha)
    for _ in range(args.warmup):
        infos, total = b.step()
        if total.status != 0:
            raise SystemExit(f"batched warm-up step failed: {total}")
    # cluster-size policy of the batched PCG (untimed; cached per device and batch)
    from simkit_gb300.autotune import tune_batch_policy, tune_pcg_variant
    policy, policy_ms = tune_batch_policy(b, use_cache=not args.retune)
    learned = None
    fb = None
    if args.learned:
        from simkit_gb300 import warmstart as ws
        net, learned = train_warm_start(args)
        fb = ws.FeatureBuilder(b, specs)
        # the warm-up steps above ran without the network: rebuild the last correction
        st = b.state()
        ut = fb.u_tilde()
        b.step()
        fb.record_correction(ut)
        del st
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    b.refresh_coarse()     # the timed steps start with fresh coarse inverses
    ranks.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0.record(stream)
    totals = []
    kept = []
    for _ in range(args.steps):
        if args.learned:
            infos, total = ws.warm_step(b, fb, net)
            kept.append(sum(i.warm_used for i in infos) / len(infos))
        else:
            infos, total = b.step()
        totals.append(total)
    ev1.record(stream)
    torch.cuda.synchronize()
    ranks.barrier()
    clock_info = clocks.stop()
    ms = ranks.max(ev0.elapsed_time(ev1))
    if any(t.status != 0 for t in totals):
        raise SystemExit(f"batched step failed: {[t.status for t in totals]}")
    inst_steps = args.instances * args.steps          # the whole batch, over all ranks
    value = inst_steps / (ms / 1000.0)
    # host gather of per-instance results (Newton iterations of the last step, final displacement)
    local = [{"newton": int(i.newton_iters), "status": int(i.status),
              "u_max": float(np.abs(b.displacement(k)).max())} for k, i in enumerate(infos)]
    gathered = gather_to_rank0(ranks.dist, shard_idx, local, args.instances)
    # one extra profiled step (phase times by CUDA events; not part of the timed region)
    b.params.profile = 1
    if args.learned:
        _, prof = ws.warm_step(b, fb, net)
    else:
        _, prof = b.step()
    b.params.profile = 0
    phase_ms = {k: getattr(prof, f"t_{k}_ms") for k in ("hessian", "assemble", "pcg", "gradient", "energy")}
    newton = ranks.sum(sum(t.newton_iters for t in totals))     # Newton iterations of the whole batch
    pcg = ranks.sum(sum(t.pcg_iters for t in totals))
    launches = ranks.sum(sum(t.launches for t in totals))
    tets = sum(sp.n_tets for sp in specs_all)
    verts = sum(sp.n_verts for sp in specs_all)
    if rank != 0:
        ranks.close()
        return 0
    # plain: the same beams one at a time (sample, state advanced to the same step count)
    rng = np.random.default_rng(1)
    sample = rng.choice(args.instances, size=min(args.plain_sample, args.instances), replace=False)
    def plain_rate(cs):
        """the sampled beams stepped one at a time through the single-instance solver"""
        ms = []
        for i in sample:
            s1 = BESolver.from_spec(specs_all[i], precision=args.precision, pcg_rtol=args.pcg_rtol, coarse=cs)
            for _ in range(args.warmup):
                s1.step()
            tune_pcg_variant(s1, use_cache=not args.retune)   # the single-instance solver at its best cluster size
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                s1.step()
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1) / args.steps)
        return 1000.0 / float(np.mean(ms))
    plain_value = plain_rate(coarse)
    # the plain form as first specified: single instance, block-Jacobi PCG
    plain_bj = plain_rate(None) if coarse is not None else plain_value
    ranks.close()
    cpu = None
    if not args.no_cpu_baseline:
        # simkit's algorithm (the oracle: spsolve, Armijo, Newton to 1e-6) on a seeded subset of
        # the beams, each stepped from rest; whole-batch rate by tet count (labelled)
        from oracle import rollout
        pick = np.random.default_rng(2).choice(args.instances, size=min(4, args.instances), replace=False)
        t_sum, tet_steps = 0.0, 0
        for i in pick:
            r = rollout.from_spec(specs_all[i])
            xc = xp = r.x_rest.copy()
            for _ in range(2):
                t0 = time.perf_counter()
                xn, _ = r.step(xc, xp)
                t_sum += time.perf_counter() - t0
                xp, xc = xc, xn
                tet_steps += specs_all[i].n_tets
        cpu = {"value": args.instances / (t_sum / tet_steps * tets), "unit": "instance-steps/s", "cores": 1,
               "kind": "port", "host": host_cpu(),
               "value_kind": "extrapolated by tet count from the measured subset",
               "sample": f"beams {sorted(int(i) for i in pick)} of the batch, 2 measured steps each from rest "
                         f"({tet_steps // 2} tets in all, {t_sum:.2f} s); whole-batch instance-steps/s = "
                         f"{args.instances} / (measured seconds per tet-step x {tets} tets)"}
    line = {
        "metric": METRIC, "value": value, "unit": "instance-steps/s", "n_gpus": n_ranks, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f32" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": f"{args.instances} beams, nx, ny in 4..16, nz in 8..48, batched "
                               + ("+ learned warm start" if args.learned else "plain Newton"),
                   "instances": args.instances, "tets": int(tets), "verts": int(verts),
                   "precision": args.precision, "pcg_rtol": args.pcg_rtol, "coarse": args.coarse,
                   "parallelism": f"instances sharded x{n_ranks} (LPT on tet count)",
                   "newton_loop": "host" if args.no_graph else "device (CUDA graph)"},
        "tet_hessians_per_s": newton / max(args.instances, 1) * tets / (ms / 1000.0),
        "newton_iters_per_instance_step": newton / inst_steps,
        "pcg_iters_per_instance_step": pcg / inst_steps,
        "gathered": {"instances": len(gathered), "failed": sum(1 for g in gathered if g["status"] != 0),
                     "newton_last_step_mean": float(np.mean([g["newton"] for g in gathered])),
                     "u_max": max(g["u_max"] for g in gathered)},
        "batch_policy": {"vec_kb": policy[0], "min_cluster": policy[1], "step_ms_by_policy": policy_ms},
        "plain_single_instance": {"value": plain_value, "unit": "instance-steps/s",
                                  "sample": f"{len(sample)} of the beams stepped alone, {args.steps} steps each"},
        "batched_over_plain": value / n_ranks / plain_value,
        "plain_single_instance_block_jacobi": {"value": plain_bj, "unit": "instance-steps/s",
                                               "sample": "the same beams, one-level block-Jacobi PCG"},
        "batched_over_plain_block_jacobi": value / n_ranks / plain_bj,
        "learned": learned,
        "warm_start_kept_fraction": float(np.mean(kept)) if kept else None,
        "cpu_baseline": cpu,
        "phase_ms_one_step": phase_ms,
        "newton_iters_profiled_step": prof.newton_iters,
        "gpu_launches": int(launches),
        "clocks": clock_info,
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--pcg-mode", type=int, default=3)
    ap.add_argument("--coarse", default="auto",
                    help="two-level PCG aggregates: none, auto, or a box size in mesh spacings")
    ap.add_argument("--coarse-refresh", default=16, type=_refresh_arg,
                    help="'step', 'newton' or k: rebuild the coarse inverse every k steps (16 measured "
                         "fastest on the 786,432-tet beam: 37.6 PCG iterations per Newton solve against "
                         "37.5 at 8 and 39.6 at 32)")
    ap.add_argument("--pcg-rtol", type=float, default=-0.1,
                    help="PCG tolerance; negative = Eisenstat-Walker forcing capped at its magnitude")
    ap.add_argument("--pcg-rtol-single", type=float, default=-0.25,
                    help="--pcg-rtol of the single-mesh headline solver (the batched and serving "
                         "modes use --pcg-rtol); with the forcing exponent 1.25, caps 0.15-0.25 measured "
                         "fastest on the 786,432-tet beam (82.6-83.2 steps/s; 0.3: 81.1, 0.1: 81.3)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the parity report of the headline line")
    ap.add_argument("--no-batched", action="store_true", help="skip the reduced batched workload of the headline line")
    ap.add_argument("--batched-coarse-refresh", default=8, type=_refresh_arg,
                    help="batched and serving workloads: rebuild the per-instance coarse inverses every k "
                         "steps (8 measured fastest on 512 beams: 4,148 instance-steps/s against 3,962 "
                         "every step, the same PCG iteration counts), every step ('step') or every Newton "
                         "iteration ('newton')")
    ap.add_argument("--ew-alpha", type=float, default=1.25,
                    help="single mesh: exponent of the Eisenstat-Walker forcing term (quarter steps over [1, 2])")
    ap.add_argument("--batched-ew-alpha", type=float, default=1.25,
                    help="batched workload: exponent of the Eisenstat-Walker forcing term")
    ap.add_argument("--no-dropin", action="store_true",
                    help="skip the timing of the drop-in backward_euler call in the headline line")
    ap.add_argument("--no-graph", action="store_true",
                    help="the host-driven Newton loop instead of the device loop (a recorded CUDA graph per step)")
    ap.add_argument("--ref-layers", type=int, default=2,
                    help="cube layers of the workload beam in the CPU reference sample (2: 12,288 tets, "
                         "about 1 s per measured step)")
    ap.add_argument("--cpu-baseline-steps", type=int, default=4,
                    help="measured CPU reference steps in the GPU arm's cpu_baseline")
    ap.add_argument("--small", action="store_true", help="use the 8x8x32 beam (quick check)")
    ap.add_argument("--retune", action="store_true", help="ignore the autotuner cache")
    ap.add_argument("--pcg-variant", type=int, default=None,
                    help="single mesh: this PCG kernel variant instead of the autotuner's choice")
    ap.add_argument("--workload", default="single", choices=["single", "batched", "serving"])
    ap.add_argument("--rate", type=float, default=2000.0, help="serving: requests per second")
    ap.add_argument("--duration", type=float, default=60.0, help="serving: seconds of traffic")
    ap.add_argument("--max-cohort", type=int, default=512)
    ap.add_argument("--max-live", type=int, default=2048)
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--plain-sample", type=int, default=16)
    ap.add_argument("--learned", action="store_true", help="batched + learned warm start")
    ap.add_argument("--train-steps", type=int, default=40)
    ap.add_argument("--epochs", type=int, default=3)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "batched":
        return run_batched(args)

    import torch
    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    ranks = Ranks("nccl")
    from simkit_gb300.beams import beam_large_jittered, beam_small_steady
    from simkit_gb300.solver import BESolver

    # replicas only: every rank runs its own instance of the workload
    spec = beam_small_steady() if args.small else beam_large_jittered(seed=replica_seed(rank))
    workload = SMALL_WORKLOAD if args.small else WORKLOAD
    coarse = None if args.coarse == "none" else (args.coarse if args.coarse == "auto" else int(args.coarse))
    solver_kw = dict(precision=args.precision, pcg_mode=args.pcg_mode, pcg_rtol=args.pcg_rtol_single,
                     coarse=coarse, coarse_refresh=args.coarse_refresh, device_loop=not args.no_graph,
                     ew_alpha=args.ew_alpha)
    solver = BESolver.from_spec(spec, **solver_kw)
    nb = solver.mesh.nb
    for _ in range(args.warmup):
        info = solver.step()
        if not info.converged:
            raise SystemExit(f"warm-up step did not converge: {info}")
    # pick the PCG kernel variant on this system (untimed; cached per device and size)
    from simkit_gb300.autotune import tune_pcg_variant
    if args.pcg_variant is None:
        variant, variant_us = tune_pcg_variant(solver, use_cache=not args.retune)
    else:
        variant, variant_us = args.pcg_variant, {}
        solver.params.pcg_variant = variant
    # the device-loop graphs of every state rotation and refresh decision, recorded before any timing
    n_plans = solver.prepare_plans()

    barrier = ranks.barrier
    stream = torch.cuda.current_stream()
    # the state the timed steps start from (the end-to-end pass replays the same steps); both passes
    # start with a fresh coarse inverse, so that they rebuild it at the same steps
    solver.refresh_coarse()
    X0 = spec.X.reshape(-1)
    x_start = ((X0 + solver.u_curr.cpu().numpy()).reshape(-1, 1), (X0 + solver.u_prev.cpu().numpy()).reshape(-1, 1))
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    torch.cuda.nvtx.range_push("timed_steps")   # lets a profiler capture exactly these steps
    infos = [solver.step() for _ in range(args.steps)]
    torch.cuda.nvtx.range_pop()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clock_info = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    ms_max = ranks.max(ms)
    for i in infos:
        if not i.converged:
            raise SystemExit(f"timed step did not converge: {i}")
    steps_total = args.steps * ws
    value = ranks.whole_job_rate(args.steps, ms_max / 1000.0)
    newton = sum(i.newton_iters for i in infos)
    pcg = sum(i.pcg_iters for i in infos)
    launches = sum(i.launches for i in infos)
    tet_hess_per_s = ws * newton * spec.n_tets / (ms_max / 1000.0)

    # profiled pass over the same number of steps (phase times by CUDA events on the launching stream)
    solver.refresh_coarse()
    solver.params.profile = 1
    pinfos = [solver.step() for _ in range(args.steps)]
    solver.params.profile = 0
    tp = {k: sum(getattr(i, f"t_{k}_ms") for i in pinfos) for k in ("hessian", "assemble", "pcg", "gradient", "energy")}
    p_newton = sum(i.newton_iters for i in pinfos)
    p_pcg = sum(i.pcg_iters for i in pinfos)
    hbm, peak_kind = peaks()
    n_coarse = 6 * solver._coarse_n_agg() if solver.coarse_form is not None else 0
    ab = algorithmic_bytes(spec, nb, n_coarse)
    pcg_ms_per_iter = tp["pcg"] / max(p_pcg, 1)
    pcg_gbs = ab["pcg_iter"] / (pcg_ms_per_iter * 1e-3) / 1e9
    hess_ms_per_launch = (tp["hessian"] + tp["assemble"]) / max(p_newton, 1)
    hess_gbs = ab["tet_hessian"] * spec.n_tets / (hess_ms_per_launch * 1e-3) / 1e9
    total_p = sum(tp.values())
    share = {k: v / total_p for k, v in tp.items()} if total_p > 0 else {}
    dominant = max(share, key=share.get) if share else "pcg"
    traffic = None
    if not args.small:   # the ncu figures are for the 32 x 32 x 128 beam
        try:
            with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
                traffic = json.load(f)
        except Exception:
            traffic = None
    if dominant in ("hessian", "assemble"):
        roof = {"bound": "hbm", "kernel": "k_tet_hessian + k_assemble", "achieved": hess_gbs, "peak": hbm,
                "unit": "GB/s", "frac": hess_gbs / hbm,
                "traffic": (traffic or {}).get("tet_hessian_bytes_per_launch"),
                "algorithmic_bytes": ab["tet_hessian"] * spec.n_tets, "ms_per_launch": hess_ms_per_launch}
    else:
        kname = {"grid": "k_pcg_grid2c (two-level grid PCG)", "cluster": "k_pcg_cluster (two-level, one cluster)"}.get(
            solver.coarse_form, "k_pcg_grid2 / k_pcg_cluster")
        roof = {"bound": "hbm", "kernel": kname + ", per PCG iteration", "achieved": pcg_gbs, "peak": hbm,
                "unit": "GB/s", "frac": pcg_gbs / hbm,
                "traffic": (traffic or {}).get("pcg2c_bytes_per_iter" if solver.coarse_form == "grid"
                                               else "pcg_bytes_per_iter" if solver.coarse_form is None else "none"),
                "algorithmic_bytes": ab["pcg_iter"], "ms_per_launch": pcg_ms_per_iter}
    roof["peak_kind"] = peak_kind
    roof["traffic_source"] = (("ncu capture committed with the repository, not measured in this run: "
                               + traffic.get("source", "profiles/")) if traffic and roof.get("traffic") else None)
    roof["phase_share"] = share
    roof["secondary"] = {"tet_hessian_assembly_gbs": hess_gbs, "tet_hessian_frac": hess_gbs / hbm,
                         "pcg_gbs": pcg_gbs, "pcg_frac": pcg_gbs / hbm}

    # end to end through the host-buffer entry point, over the same steps as the timed region
    # three rotating pinned host buffers: the new positions never overwrite x_curr or x_prev
    bufs = [torch.empty(x_start[0].shape, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    # one untimed host-buffer step (first-call pinned staging allocation)
    solver.step_host(x_start[0], x_start[1], out=bufs[2])
    bufs[0][...] = x_start[0]
    bufs[1][...] = x_start[1]
    x_curr, x_prev = bufs[0], bufs[1]
    solver.refresh_coarse()
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        free = next(b for b in bufs if not np.shares_memory(b, x_curr) and not np.shares_memory(b, x_prev))
        x_next, info = solver.step_host(x_curr, x_prev, out=free)
        x_prev, x_curr = x_curr, x_next
    torch.cuda.synchronize()
    barrier()
    e2e_s = ranks.max(time.perf_counter() - t0)
    e2e = {"value": ranks.whole_job_rate(args.steps, e2e_s), "unit": "steps/s", "h2d_bytes_per_step": 2 * 3 * spec.n_verts * 8,
           "d2h_bytes_per_step": 3 * spec.n_verts * 8}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the same measurement the reference arm makes (real slab steps), over a few steps
        ref = (CpuReferenceSteps(spec, layers=spec.dims[0], restart=10 ** 9) if args.small
               else CpuReferenceSteps(spec, layers=args.ref_layers))
        for _ in range(args.cpu_baseline_steps):
            ref.step()
        sm = ref.summary(skip=1)
        cpu = {"value": sm["extrapolated_steps_per_s"], "unit": "steps/s", "cores": 1, "kind": "port",
               "sample": sm["sample"], "value_kind": "extrapolated from the measured slab steps (upper bound)",
               "measured": sm, "host": host_cpu()}

    parity = None
    if rank == 0 and not args.small and not args.no_parity:
        parity = parity_report(spec, solver_kw)
    batched = None
    if rank == 0 and not args.small and not args.no_batched:
        batched = batched_summary(coarse_refresh=args.batched_coarse_refresh)
    dropin = None
    if rank == 0 and not args.small and not args.no_dropin:
        dropin = dropin_summary(cpu_steps=0 if args.no_cpu_baseline else 2)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision == "mixed" else "f64",
            "data": "synthetic",
            "config": {"workload": workload, "tets": spec.n_tets, "verts": spec.n_verts, "blocks": nb,
                       "precision": args.precision, "pcg_mode": args.pcg_mode, "pcg_rtol": args.pcg_rtol_single,
                       "pcg_variant": variant, "pcg_variant_us_per_iter": variant_us,
                       "newton_loop": "device (one CUDA graph per step)" if n_plans else "host",
                       "ew_alpha": args.ew_alpha,
                       "coarse_box": solver.coarse_box, "coarse_refresh": args.coarse_refresh,
                       "tol": 1e-6, "parallelism": f"replicas x{ws}", "l2": "inputs larger than L2, no flush"},
            "tet_hessians_per_s": tet_hess_per_s,
            "newton_iters_per_step": newton / args.steps,
            "pcg_iters_per_newton": pcg / max(newton, 1),
            "pcg_iters_timed": pcg,
            "gpu_launches": launches,
            "e2e": e2e,
            "roofline": roof,
            "cpu_baseline": cpu,
            "parity": parity,
            "batched": batched,
            "dropin": dropin,
            "clocks": clock_info,
        }
        print(json.dumps(line))
    ranks.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
