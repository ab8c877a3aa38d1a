"""Checkpoint and resume of device rollouts and of the warm-start network.

A rollout is resumable from its displacement history: the backward-Euler state is (u at step k,
u at step k-1), BDF2's adds k-2 and k-3, plus the step counter and the seed that drew the workload.
The warm-start network resumes from its FP32 master weights and biases with Adam's moments and step
count (the BF16 copies the GEMMs read are derived from the masters on load).  The two-level PCG's
coarse inverse is not stored: a resumed ``BESolver`` rebuilds it at its first step, so with
``coarse_refresh=k > 1`` the resumed steps agree with uninterrupted ones to the Newton tolerance
(bitwise with a rebuild every step).  Both go to one ``.npz``
file per checkpoint (numpy arrays; no pickled objects), written to a temporary name and renamed, so
an interrupted write never leaves a truncated checkpoint behind.

simkit has no checkpointing of its own beyond its result cache
(``simkit/filesystem/compute_with_cache_check.py``, mirrored in ``rollout_io``).
"""

from __future__ import annotations

import os

import numpy as np
import torch

FORMAT = 1


def _write(path, arrays):
    tmp = f"{path}.tmp.{os.getpid()}.npz"
    np.savez(tmp, **arrays)
    os.replace(tmp, path)


def save_rollout(path, solver, seed=None):
    """The solver's displacement history and step count (a ``BESolver`` or ``BatchedBESolver``)."""
    levels = [solver.u_curr, solver.u_prev]
    if solver.integrator == "bdf2":
        levels += [solver.u_prev2, solver.u_prev3]
    arrays = {f"u{k}": t.detach().cpu().numpy() for k, t in enumerate(levels)}
    arrays.update(format=np.int64(FORMAT), kind=np.array("rollout"), integrator=np.array(solver.integrator),
                  steps=np.int64(solver.steps), n_dof=np.int64(levels[0].numel()),
                  seed=np.int64(-1 if seed is None else seed))
    _write(path, arrays)


def load_rollout(path, solver):
    """Restore a rollout checkpoint into a solver built for the same mesh; returns the stored seed
    (None if none was stored).  Raises ValueError on a mismatch of kind, integrator or size."""
    with np.load(path, allow_pickle=False) as d:
        if int(d["format"]) != FORMAT or str(d["kind"]) != "rollout":
            raise ValueError(f"{path} is not a rollout checkpoint of format {FORMAT}")
        if str(d["integrator"]) != solver.integrator:
            raise ValueError(f"checkpoint integrator {d['integrator']} != solver's {solver.integrator}")
        if int(d["n_dof"]) != solver.u_curr.numel():
            raise ValueError(f"checkpoint has {int(d['n_dof'])} DOFs, the solver {solver.u_curr.numel()}")
        levels = [torch.from_numpy(d[f"u{k}"]) for k in range(4 if solver.integrator == "bdf2" else 2)]
        steps = int(d["steps"])
        seed = int(d["seed"])
    if hasattr(solver, "inst_rows"):   # BatchedBESolver: one tuple of levels
        solver.set_state(tuple(t.to(solver.u_curr.device) for t in levels))
    else:                              # BESolver: the levels as arguments
        solver.set_state(*levels)
    solver.steps = steps
    return None if seed < 0 else seed


def save_network(path, net):
    """A ``warmstart.WarmStartMLP``: FP32 master weights and biases, Adam moments and step."""
    arrays = {"format": np.int64(FORMAT), "kind": np.array("warmstart"), "t": np.int64(net.t),
              "lr": np.float64(net.lr), "layers": np.int64(len(net.W))}
    for li in range(len(net.W)):
        for name, seq in (("W", net.W), ("b", net.b), ("mW", net.mW), ("vW", net.vW), ("mb", net.mb),
                          ("vb", net.vb)):
            arrays[f"{name}{li}"] = seq[li].detach().cpu().numpy()
    _write(path, arrays)


def load_network(path, net):
    """Restore a network checkpoint into a ``WarmStartMLP`` of the same shape (BF16 copies rebuilt)."""
    with np.load(path, allow_pickle=False) as d:
        if int(d["format"]) != FORMAT or str(d["kind"]) != "warmstart":
            raise ValueError(f"{path} is not a warm-start checkpoint of format {FORMAT}")
        if int(d["layers"]) != len(net.W):
            raise ValueError("layer count differs")
        for li in range(len(net.W)):
            for name, seq in (("W", net.W), ("b", net.b), ("mW", net.mW), ("vW", net.vW), ("mb", net.mb),
                              ("vb", net.vb)):
                src = torch.from_numpy(d[f"{name}{li}"])
                if tuple(src.shape) != tuple(seq[li].shape):
                    raise ValueError(f"{name}{li}: shape {tuple(src.shape)} != {tuple(seq[li].shape)}")
                seq[li].copy_(src)
        net.t = int(d["t"])
        net.lr = float(d["lr"])
    net.refresh_bf16()
