"""Instance sharding of one batch across ranks (one process per GPU).

Batched instances are independent meshes, so a batch splits across GPUs with
no exchange in the solve: every rank steps its share of the instances and the
per-instance results are gathered on the host of rank 0 at the end.  The
split is longest-processing-time-first bin packing on tet count (a step's
work is close to linear in the tets of each instance): instances in
decreasing size, each to the rank with the least work so far, ties to the
lowest rank.  LPT keeps the largest rank's load within 4/3 of the optimum,
and within one instance of the mean.

simkit has no multi-process path; its user loops call ``backward_euler`` per
mesh (``simkit/integrators/backward_euler.py:27``).
"""

from __future__ import annotations

import heapq

import numpy as np


def lpt_partition(weights, n_parts: int):
    """Indices of ``weights`` per part (each list in increasing index order) by LPT bin packing."""
    w = np.asarray(weights, dtype=np.float64).ravel()
    if n_parts < 1:
        raise ValueError("n_parts must be >= 1")
    if np.any(w < 0):
        raise ValueError("weights must be non-negative")
    order = sorted(range(w.size), key=lambda i: (-w[i], i))
    heap = [(0.0, p) for p in range(n_parts)]
    parts = [[] for _ in range(n_parts)]
    for i in order:
        load, p = heapq.heappop(heap)
        parts[p].append(i)
        heapq.heappush(heap, (load + w[i], p))
    return [sorted(p) for p in parts]


def part_loads(weights, parts):
    w = np.asarray(weights, dtype=np.float64).ravel()
    return np.array([w[p].sum() for p in parts])


def shard(specs, rank: int, world: int):
    """(global indices, specs) of this rank's instances: LPT by tet count over ``world`` ranks."""
    parts = lpt_partition([s.n_tets for s in specs], world)
    idx = parts[rank]
    return idx, [specs[i] for i in idx]


def gather_to_rank0(dist, idx, local_results, n_total: int):
    """Per-instance results of every rank, in global instance order, on rank 0 (None elsewhere).
    ``dist`` is ``torch.distributed`` (or None for one process); ``local_results[k]`` belongs to
    global instance ``idx[k]``; results are host objects (picklable)."""
    pairs = list(zip(idx, local_results))
    if dist is None:
        gathered = [pairs]
        rank = 0
    else:
        rank = dist.get_rank()
        gathered = [None] * dist.get_world_size() if rank == 0 else None
        dist.gather_object(pairs, gathered, dst=0)
    if rank != 0:
        return None
    out = [None] * n_total
    seen = 0
    for part in gathered:
        for i, r in part:
            if out[i] is not None:
                raise RuntimeError(f"instance {i} reported by two ranks")
            out[i] = r
            seen += 1
    if seen != n_total:
        raise RuntimeError(f"gathered {seen} of {n_total} instances")
    return out
