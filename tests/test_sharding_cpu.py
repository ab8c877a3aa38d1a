"""Instance sharding of one batch across ranks (LPT on tet count) and the host gather of per-instance
results, on CPU: partition properties, and two gloo ranks (127.0.0.1) that each step their share of a
batch of small beams with the FP64 oracle and gather to rank 0, which must equal one process stepping
the whole batch."""

import os
import socket

import numpy as np
import pytest

from simkit_gb300.sharding import gather_to_rank0, lpt_partition, part_loads, shard


def test_lpt_partition_covers_every_instance_once_and_balances():
    rng = np.random.default_rng(0)
    for world in (1, 2, 3, 8):
        w = rng.integers(768, 73728, size=512)
        parts = lpt_partition(w, world)
        allidx = np.concatenate([np.asarray(p, dtype=np.int64) for p in parts])
        assert np.array_equal(np.sort(allidx), np.arange(w.size))
        loads = part_loads(w, parts)
        assert loads.max() <= w.sum() / world + w.max()
        assert loads.max() / loads.mean() < 1.01           # 512 instances: near perfect balance


def test_lpt_partition_is_within_four_thirds_of_optimal_on_small_cases():
    import itertools
    rng = np.random.default_rng(1)
    for _ in range(30):
        w = rng.integers(1, 20, size=7)
        best = min(max(sum(w[i] for i in range(7) if a[i] == p) for p in range(3))
                   for a in itertools.product(range(3), repeat=7))
        got = part_loads(w, lpt_partition(w, 3)).max()
        assert got <= 4.0 / 3.0 * best + 1e-9


def test_lpt_partition_is_deterministic_and_rejects_bad_input():
    w = [5, 5, 5, 5, 1]
    assert lpt_partition(w, 2) == lpt_partition(w, 2) == [[0, 2, 4], [1, 3]]
    with pytest.raises(ValueError):
        lpt_partition(w, 0)
    with pytest.raises(ValueError):
        lpt_partition([1, -1], 2)


def _specs():
    from simkit_gb300.beams import beam_batch
    return beam_batch(7, seed=11, nx_range=(2, 4), ny_range=(1, 2), nz_range=(2, 4))


def _step_result(spec):
    """Per-instance result of two backward-Euler steps from rest with the FP64 oracle."""
    from oracle import rollout
    r = rollout.from_spec(spec)
    xc = xp = r.x_rest.copy()
    iters = []
    for _ in range(2):
        xn, info = r.step(xc, xp)
        xp, xc = xc, xn
        iters.append(info.iters)
    return {"iters": iters, "u": (xc - r.x_rest).ravel().copy()}


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    try:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        specs = _specs()
        idx, mine = shard(specs, rank, world)
        results = [_step_result(s) for s in mine]
        out = gather_to_rank0(dist, idx, results, len(specs))
        dist.barrier()
        dist.destroy_process_group()
        q.put((rank, idx, out, None))
    except Exception as e:  # reported to the parent, which fails the test
        q.put((rank, None, None, repr(e)))


def test_two_gloo_ranks_gather_equals_single_process_batch():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = {}
    try:
        for _ in range(2):
            rank, idx, out, err = q.get(timeout=240)
            assert err is None, f"rank {rank}: {err}"
            got[rank] = (idx, out)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs)
    specs = _specs()
    assert sorted(got[0][0] + got[1][0]) == list(range(len(specs)))
    assert got[1][1] is None                         # only rank 0 holds the gathered batch
    single = gather_to_rank0(None, list(range(len(specs))), [_step_result(s) for s in specs], len(specs))
    for a, b in zip(got[0][1], single):
        assert a["iters"] == b["iters"]
        assert np.array_equal(a["u"], b["u"])
