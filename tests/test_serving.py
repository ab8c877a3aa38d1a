"""Serving loop: device pattern construction and cohort assembly against the host
pattern builder (CPU), and a short served stream against the batched solver built
from the same beams (GPU)."""

import ctypes

import numpy as np
import pytest
import torch

from simkit_gb300.beams import beam_mesh


def _host_pattern(T, n):
    from simkit_gb300 import _lib
    lib = _lib.load()
    T = np.ascontiguousarray(T.astype(np.int32))
    t = T.shape[0]
    nb = ctypes.c_int64(0)
    Tp = T.ctypes.data_as(ctypes.c_void_p)
    assert lib.skg_pattern_build(Tp, n, t, ctypes.byref(nb), None, None, None, None, None, None, None) == 0
    nb = nb.value
    arrs = [np.empty(k, np.int32) for k in (n + 1, nb, n, nb + 1, 16 * t, n + 1, 4 * t)]
    a = lambda x: x.ctypes.data_as(ctypes.c_void_p)
    assert lib.skg_pattern_build(Tp, n, t, ctypes.byref(ctypes.c_int64(0)), *[a(x) for x in arrs]) == 0
    rowptr, col, diag, hc_ptr, hc_src, v2t_ptr, v2t = arrs
    row = np.repeat(np.arange(n, dtype=np.int32), np.diff(rowptr))
    return rowptr, col, diag, row, hc_ptr, hc_src, v2t_ptr, v2t


def test_device_pattern_matches_host_builder():
    from simkit_gb300.mesh import device_pattern
    X1, T1 = beam_mesh(3, 4, 5)
    X2, T2 = beam_mesh(2, 2, 3)
    T = np.concatenate([T1, T2 + X1.shape[0]])
    n = X1.shape[0] + X2.shape[0]
    T = T[np.random.default_rng(0).permutation(T.shape[0])]
    ref = _host_pattern(T, n)
    got = device_pattern(torch.from_numpy(T.astype(np.int32)), n)
    for r, g in zip(ref, got):
        assert np.array_equal(r, g.numpy())


def test_device_pattern_rejects_isolated_vertices():
    from simkit_gb300.mesh import device_pattern
    _, T = beam_mesh(1, 1, 1)
    with pytest.raises(ValueError):
        device_pattern(torch.from_numpy(T.astype(np.int32)), 9)


def test_concatenated_patterns_equal_pattern_of_concatenation():
    from simkit_gb300.mesh import device_pattern
    from simkit_gb300.serving import concat_patterns
    shapes = [(2, 3, 4), (4, 2, 2), (1, 1, 5), (3, 3, 3)]
    parts, Ts, n_off, t_off, b_off = [], [], [0], [0], [0]
    for d in shapes:
        X, T = beam_mesh(*d)
        p = device_pattern(torch.from_numpy(T.astype(np.int32)), X.shape[0])
        parts.append(p)
        Ts.append(T + n_off[-1])
        n_off.append(n_off[-1] + X.shape[0])
        t_off.append(t_off[-1] + T.shape[0])
        b_off.append(b_off[-1] + p[1].numel())
    got = concat_patterns(parts, n_off[:-1], t_off[:-1], b_off[:-1], b_off[-1], t_off[-1])
    ref = _host_pattern(np.concatenate(Ts), n_off[-1])
    for r, g in zip(ref, got):
        assert np.array_equal(r, g.numpy())


def test_beam_meshes_equal_single_beams():
    from simkit_gb300.beams import beam_meshes
    dims = [(4, 5, 9), (16, 16, 48), (7, 4, 8), (1, 1, 1)]
    X, T, vo, to = beam_meshes(dims)
    for s, d in enumerate(dims):
        Xs, Ts = beam_mesh(*d)
        assert np.array_equal(X[vo[s]:vo[s + 1]], Xs)
        assert np.array_equal(T[to[s]:to[s + 1]], Ts + vo[s])


def test_request_stream_is_a_seeded_poisson_stream():
    from simkit_gb300.serving import request_stream
    a = request_stream(200.0, 5.0, seed=3)
    b = request_stream(200.0, 5.0, seed=3)
    assert [r.dims for r in a] == [r.dims for r in b]
    t = np.array([r.t_arrival for r in a])
    assert np.all(np.diff(t) >= 0) and t[-1] < 5.0
    assert abs(len(a) - 1000) < 5 * np.sqrt(1000)
    d = np.array([r.dims for r in a])
    assert d[:, 0].min() >= 4 and d[:, 0].max() <= 16 and d[:, 2].min() >= 8 and d[:, 2].max() <= 48
    g = np.array([r.gravity for r in a])
    assert np.allclose(np.linalg.norm(g, axis=1), 9.8)


@pytest.mark.gpu
@pytest.mark.parametrize("coarse", [False, True])
def test_cohort_steps_equal_batched_solver_from_specs(coarse):
    """A cohort assembled on the device from shape templates takes bitwise the same
    steps as the batched solver built from the equivalent beam specs on the host, with
    and without the per-instance two-level data (template pieces concatenated with shifts
    on the device vs aggregates built for the batch on the host)."""
    from simkit_gb300.batched import BatchedBESolver
    from simkit_gb300.beams import make_beam
    from simkit_gb300.serving import BeamRequest, TemplateCache, build_cohort
    rng = np.random.default_rng(4)
    reqs = []
    for i, d in enumerate([(4, 5, 9), (6, 4, 12), (4, 5, 9)]):
        g = rng.standard_normal(3)
        g = 9.8 * g / np.linalg.norm(g)
        reqs.append(BeamRequest(i, d, float(np.exp(rng.uniform(np.log(1e5), np.log(1e7)))),
                                float(rng.uniform(0.3, 0.49)), g, 3, 0.0))
    cache = TemplateCache("cuda", coarse=coarse)   # both shapes in one chunk: one has nonzero bases
    a, _ = build_cohort(cache, reqs)
    assert len(cache.shapes) == 2 and max(tp.tbase for tp in cache.shapes.values()) > 0
    b = BatchedBESolver([make_beam(*r.dims, cell=0.025, ym=r.ym, pr=r.pr, rho=1000.0, gravity=r.gravity)
                         for r in reqs], coarse="auto" if coarse else None)
    assert (a.mesh.c.coarse is not None and bool(a.mesh.c.coarse)) == coarse
    for _ in range(3):
        ia, ta = a.step()
        ib, tb = b.step()
        assert ta.status == 0 and tb.status == 0
        assert [i.newton_iters for i in ia] == [i.newton_iters for i in ib]
        assert torch.equal(a.u_curr, b.u_curr)


@pytest.mark.gpu
def test_short_stream_is_served():
    from simkit_gb300.serving import BeamServer, request_stream
    reqs = request_stream(40.0, 1.5, steps=3, seed=9, nx_range=(4, 6), ny_range=(4, 6), nz_range=(8, 12))
    srv = BeamServer(max_cohort=64, max_live=256, hbm_reserve_gb=1.0)
    st = srv.run(reqs, 1.5, serve_backlog=True)
    s = st.summary()
    assert st.completed == st.admitted == st.arrived == len(reqs)
    assert st.failed_steps == 0 and st.backlog == 0
    assert all(r.t_done >= r.t_admit >= r.t_arrival for r in reqs)
    assert s["latency_ms_p99"] >= s["latency_ms_p50"] > 0


def test_admission_refuses_requests_beyond_free_hbm(monkeypatch):
    """Admission takes requests, oldest first, while the free HBM less the reserve covers their
    estimated footprint; with the reserve above the free memory nothing is admitted and the
    requests stay queued (CPU: the free-memory query is replaced by a fake)."""
    import collections
    from simkit_gb300.serving import BeamRequest, BeamServer
    free = {"bytes": 8 * 2 ** 30}
    monkeypatch.setattr(torch.cuda, "mem_get_info", lambda *a: (free["bytes"], 16 * 2 ** 30))
    reqs = [BeamRequest(i, (4, 4, 8), 1e6, 0.4, np.array([0.0, -9.8, 0.0]), 10, 0.0) for i in range(5)]
    srv = BeamServer(max_cohort=64, max_live=256, hbm_reserve_gb=1.0, device="cpu")
    srv.bytes_per_tet = 2 ** 20                     # 768 MiB per 768-tet request
    pending = collections.deque(reqs)
    take = srv._admit(pending, 0)                   # 7 GiB usable: nine would fit, five are queued
    assert [r.rid for r in take] == [0, 1, 2, 3, 4] and not pending
    pending = collections.deque(reqs)
    free["bytes"] = int(2.6 * 2 ** 30)              # 1.6 GiB usable: two requests
    take = srv._admit(pending, 0)
    assert [r.rid for r in take] == [0, 1] and [r.rid for r in pending] == [2, 3, 4]
    srv.reserve = 64 * 2 ** 30                      # reserve above the free memory: refuse all
    pending = collections.deque(reqs)
    assert srv._admit(pending, 0) == [] and len(pending) == 5
    srv.reserve = 0
    free["bytes"] = 8 * 2 ** 30
    assert len(srv._admit(collections.deque(reqs), 252)) == 4       # max_live caps the cohort too


@pytest.mark.gpu
def test_server_with_no_free_hbm_queues_every_request():
    """With a reserve larger than the GPU's memory the server admits nothing: every request is
    reported as backlog, none fails, and no cohort is built."""
    from simkit_gb300.serving import BeamServer, request_stream
    reqs = request_stream(40.0, 0.5, steps=2, seed=2, nx_range=(4, 5), ny_range=(4, 5), nz_range=(8, 9))
    srv = BeamServer(max_cohort=64, max_live=256, hbm_reserve_gb=1.0e6)
    st = srv.run(reqs, 0.5)
    assert st.admitted == 0 and st.completed == 0 and st.cohorts == 0
    assert st.backlog == st.arrived == len(reqs) and st.failed_steps == 0
