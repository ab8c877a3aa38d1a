"""Trajectory files of device rollouts, in simkit's cache format.

simkit caches computed results with ``compute_with_cache_check``
(``simkit/filesystem/compute_with_cache_check.py:4-48``): the outputs of a
function are stored with ``np.savez`` under keys ``v0, v1, ...`` and read back
in key order, each entry converted to a Python scalar where it is one
(``.item()``) and kept as an array otherwise.  ``compute_with_cache_check``
below keeps that contract, so caches written by either side read the same on
the other, and ``cached_rollout`` stores a device rollout in it: positions
(steps + 1, n, 3), Newton iterations and final relative residuals per step.
"""

from __future__ import annotations

import numpy as np


def compute_with_cache_check(func, cache_path, read_cache: bool = True):
    """Results of ``func()`` as a tuple, read from the ``.npz`` cache when it exists (and
    ``read_cache``), else computed and written there (simkit's keys v0, v1, ...)."""
    if read_cache:
        try:
            data = np.load(cache_path, allow_pickle=True)
            out = ()
            for key in sorted(data.files, key=lambda s: int(s[1:])):
                value = data[key]
                try:
                    out += (value.item(),)
                except ValueError:
                    out += (value,)
            return out
        except Exception:
            print(f"rollout cache {cache_path} unreadable; computing the result")
    else:
        print(f"rollout cache reading off; computing the result into {cache_path}")
    output = func()
    if not isinstance(output, tuple):
        output = (output,)
    np.savez(cache_path, **{f"v{i}": arg for i, arg in enumerate(output)})
    return output


def rollout_trajectory(solver, steps: int):
    """Run ``steps`` steps of a ``BESolver`` (or a one-instance ``BatchedBESolver``) and return
    (positions (steps + 1, n, 3) float64, newton iterations (steps,), residuals (steps,)) on the host;
    positions are rest + displacement, the first row the state before the first step."""
    X = solver.mesh.X.detach().cpu().numpy().reshape(-1, 3)
    traj = [X + solver.u_curr.cpu().numpy().reshape(-1, 3)]
    iters, res = [], []
    for _ in range(steps):
        info = solver.step()
        if isinstance(info, tuple):          # batched: (per-instance infos, total)
            info = info[1]
        iters.append(info.newton_iters)
        res.append(info.residual)
        traj.append(X + solver.u_curr.cpu().numpy().reshape(-1, 3))
    return np.stack(traj), np.array(iters, dtype=np.int64), np.array(res, dtype=np.float64)


def cached_rollout(solver, steps: int, cache_path, read_cache: bool = True):
    """``rollout_trajectory`` through the cache: a second call with the same path reads the file."""
    return compute_with_cache_check(lambda: rollout_trajectory(solver, steps), cache_path, read_cache)
