"""Replica bookkeeping of ``bench.py`` under two ranks on CPU (gloo, 127.0.0.1).

The multi-GPU form of this path is replicas only: every rank steps its own
independent meshes and the process group carries nothing but the barriers
around the timed region and the max-over-ranks time.  Checked here with
world size 2: the ranks draw different workloads, the reduced time is the
slowest rank's, the whole-job rate counts every rank's units, and the two
arms' rank bookkeeping (single mesh, batched) agree with that.
"""

import importlib.util
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    try:
        bench = _load_bench()
        from simkit_gb300.beams import beam_batch
        r = bench.Ranks("gloo")
        specs = beam_batch(3, seed=bench.replica_seed(r.rank))
        digest = [float(s.X.sum()) for s in specs] + [float(s.mu.sum()) for s in specs]
        r.barrier()
        ms = 10.0 + 7.5 * r.rank          # rank 1 is the slow one
        ms_max = r.max(ms)
        rate = r.whole_job_rate(8, ms_max / 1000.0)
        r.barrier()
        r.close()
        q.put((rank, r.ws, digest, ms_max, rate, None))
    except Exception as e:  # reported to the parent, which fails the test
        q.put((rank, None, None, None, None, repr(e)))


def test_two_gloo_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    try:
        for _ in range(2):
            rank, world, digest, ms_max, rate, err = q.get(timeout=240)
            assert err is None, f"rank {rank}: {err}"
            out[rank] = (world, digest, ms_max, rate)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert sorted(out) == [0, 1]
    assert all(o[0] == 2 for o in out.values())
    # independent replicas: different seeded draws of the workload
    assert out[0][1] != out[1][1]
    # max over ranks, seen identically by both
    assert out[0][2] == out[1][2] == pytest.approx(17.5)
    # whole job: 2 ranks x 8 units over the slowest rank's 17.5 ms
    assert out[0][3] == pytest.approx(16 / 0.0175)
    assert all(p.exitcode == 0 for p in procs)


def test_single_rank_defaults(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    bench = _load_bench()
    r = bench.Ranks("gloo")
    assert (r.ws, r.rank, r.local) == (1, 0, 0)
    assert r.dist is None
    assert r.max(3.25) == 3.25
    assert r.whole_job_rate(10, 2.0) == 5.0
    assert bench.replica_seed(0) == 0
    r.close()
