"""Autotuners for the PCG kernels.

Single systems: the grid-persistent PCG kernel comes in variants that trade lanes per block row (G) against
block rows in flight per lane group (U): (8,1), (16,1), (8,2), (16,2),
(4,2), (4,4), (2,4), (8,4), (2,2).  Which one keeps the most loads in flight without idling lanes
depends on the row lengths of the mesh and on the device, so the variant is
picked by timing: each candidate runs one backward-Euler step from the same
saved state with per-phase CUDA-event timing, and the variant with the
lowest PCG time over the step wins (the variants round differently, so their
iteration counts differ a little; the per-iteration times are reported).  The
two-level grid kernel also comes with two grid barriers per iteration instead of
three (the coarse residual carried by a recurrence), in three shapes.  Results are cached in a JSON file keyed
by device, system size and precision (``$SIMKIT_GB300_CACHE`` or
``~/.cache/simkit_gb300/autotune.json``).  Systems small enough for one
thread-block cluster have one knob instead, the cluster size (16, 8, 4 or 2
CTAs: fewer CTAs make the cluster barriers cheaper and give each CTA more rows).

Batches: the cluster-size policy of the batched PCG (the per-CTA shared-memory
cap for vectors and the smallest cluster an instance gets) decides how many
instances solve at once and whether their block records stay in shared
memory; candidates are timed over one whole batched step from the same saved
state, and the fastest is cached by device, instance count, total rows and
precision.
"""

from __future__ import annotations

import json
import os

import torch

VARIANTS = {0: (8, 1), 1: (16, 1), 2: (8, 2), 3: (16, 2), 4: (4, 2), 5: (4, 4), 6: (2, 4), 7: (8, 4), 8: (2, 2)}
# two-level grid PCG with two barriers per iteration (coarse residual by recurrence), 768-thread blocks
TWO_BARRIER_VARIANTS = {18: (4, 2), 19: (8, 2), 20: (2, 2)}
CLUSTER_ROWS = 24576  # systems up to this size use the one-cluster PCG (no variants)


def _cache_path():
    base = os.environ.get("SIMKIT_GB300_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "simkit_gb300"))
    return os.path.join(base, "autotune.json")


def _load():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except Exception:
        return {}


def _store(table):
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
    except OSError:
        pass


def _key(solver):
    bucket = 1 << max(0, int(solver.mesh.n - 1).bit_length())
    coarse = getattr(solver, "coarse_box", None)
    return (f"{torch.cuda.get_device_name()}|rows<={bucket}|prec={solver.precision}|mode={solver.params.pcg_mode}"
            f"|coarse={coarse}")


def _history(solver):
    """The solver's displacement levels (current first)."""
    levels = [solver.u_curr, solver.u_prev]
    if getattr(solver, "integrator", "be") == "bdf2":
        levels += [solver.u_prev2, solver.u_prev3]
    return levels


CLUSTER_VARIANTS = {1: 16, 2: 8, 3: 4, 4: 2}   # thread-block cluster sizes of the one-cluster PCG


def tune_pcg_variant(solver, variants=None, use_cache=True):
    """Pick the fastest PCG kernel variant for ``solver``: the (lanes per row, rows in flight)
    variant of the grid kernel, or the cluster size of the one-cluster kernel; returns
    (variant, timings_us per PCG iteration)."""
    mode = solver.params.pcg_mode
    cluster = mode == 2 or (mode == 3 and solver.mesh.n <= CLUSTER_ROWS)
    if mode not in (1, 2, 3, 5, 7):
        return solver.params.pcg_variant, {}
    if variants is None:
        two_level_grid = getattr(solver, "coarse_form", None) == "grid" and not cluster
        variants = (tuple(CLUSTER_VARIANTS) if cluster
                    else tuple(VARIANTS) + tuple(v + 9 for v in VARIANTS) + tuple(TWO_BARRIER_VARIANTS)
                    if two_level_grid else tuple(VARIANTS))
    key = _key(solver)
    table = _load() if use_cache else {}
    if key in table:
        solver.params.pcg_variant = int(table[key]["variant"])
        return solver.params.pcg_variant, table[key]["us_per_iter"]
    hist = [t.clone() for t in _history(solver)]
    steps = solver.steps
    old_profile = solver.params.profile
    timings = {}
    totals = {}
    for v in variants:
        for dst, src in zip(_history(solver), hist):
            dst.copy_(src)
        solver.params.pcg_variant = v
        solver.params.profile = 1
        info = solver.step()
        timings[v] = 1e3 * info.t_pcg_ms / max(info.pcg_iters, 1)
        totals[v] = info.t_pcg_ms
    for dst, src in zip(_history(solver), hist):
        dst.copy_(src)
    solver.steps = steps
    solver.params.profile = old_profile
    # the whole step's PCG time decides: the forms do not round alike, so their iteration counts differ a little
    best = min(totals, key=totals.get)
    solver.params.pcg_variant = best
    if use_cache:
        table[key] = {"variant": best, "us_per_iter": {str(k): v for k, v in timings.items()}}
        _store(table)
    return best, timings


BATCH_POLICIES = ((60, 1), (60, 4), (170, 1), (170, 4), (220, 4))  # (vector KiB cap, smallest cluster)


def _batch_key(bsolver):
    return (f"{torch.cuda.get_device_name()}|batch={bsolver.n_inst}|rows={bsolver.mesh.n}"
            f"|prec={bsolver.precision}")


def tune_batch_policy(bsolver, policies=BATCH_POLICIES, use_cache=True):
    """Pick the batched PCG cluster policy for ``bsolver`` (a BatchedBESolver) by timing one
    step per candidate from the same state; returns ((vec_kb, min_cluster), timings_ms)."""
    key = _batch_key(bsolver)
    table = _load() if use_cache else {}
    if key in table:
        vk, mc = table[key]["policy"]
        bsolver.params.batch_vec_kb, bsolver.params.batch_min_cluster = int(vk), int(mc)
        return (int(vk), int(mc)), table[key]["ms"]
    st = bsolver.state()
    steps = bsolver.steps
    age = getattr(bsolver, "_coarse_age", None)   # every candidate step takes the same refresh decision
    timings = {}
    stream = torch.cuda.current_stream()
    for vk, mc in policies:
        bsolver.params.batch_vec_kb, bsolver.params.batch_min_cluster = vk, mc
        best = None
        for _ in range(2):
            bsolver.set_state(st)
            bsolver._coarse_age = age
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            bsolver.step()
            e1.record(stream)
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1)
            best = t if best is None else min(best, t)
        timings[f"{vk},{mc}"] = best
    bsolver.set_state(st)
    bsolver.steps = steps
    bsolver._coarse_age = age
    vk, mc = map(int, min(timings, key=timings.get).split(","))
    bsolver.params.batch_vec_kb, bsolver.params.batch_min_cluster = vk, mc
    if use_cache:
        table[key] = {"policy": [vk, mc], "ms": timings}
        _store(table)
    return (vk, mc), timings
