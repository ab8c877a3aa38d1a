"""Checkpoint / resume: a rollout interrupted and resumed from its checkpoint takes bitwise the same
steps as one that ran through (GPU); the network checkpoint restores weights, Adam moments and step
(GPU); format checks and refused mismatches (CPU)."""

import numpy as np
import pytest
import torch


class _FakeSolver:
    """Host stand-in with the attributes the rollout checkpoint reads and writes."""

    def __init__(self, n, integrator="be"):
        self.integrator = integrator
        self.u_curr = torch.zeros(3 * n, dtype=torch.float64)
        self.u_prev = torch.zeros(3 * n, dtype=torch.float64)
        self.u_prev2 = torch.zeros(3 * n, dtype=torch.float64) if integrator == "bdf2" else None
        self.u_prev3 = torch.zeros(3 * n, dtype=torch.float64) if integrator == "bdf2" else None
        self.steps = 0

    def set_state(self, u_curr, u_prev, u_prev2=None, u_prev3=None):
        self.u_curr.copy_(torch.as_tensor(u_curr))
        self.u_prev.copy_(torch.as_tensor(u_prev))
        if self.integrator == "bdf2":
            self.u_prev2.copy_(torch.as_tensor(u_prev2))
            self.u_prev3.copy_(torch.as_tensor(u_prev3))


@pytest.mark.parametrize("integrator", ["be", "bdf2"])
def test_rollout_checkpoint_round_trip_on_host(tmp_path, integrator):
    from simkit_gb300.checkpoint import load_rollout, save_rollout
    a = _FakeSolver(7, integrator)
    g = torch.Generator().manual_seed(0)
    for t in (a.u_curr, a.u_prev, a.u_prev2, a.u_prev3):
        if t is not None:
            t.copy_(torch.randn(t.shape, generator=g, dtype=torch.float64))
    a.steps = 11
    path = tmp_path / "ck.npz"
    save_rollout(path, a, seed=5)
    b = _FakeSolver(7, integrator)
    assert load_rollout(path, b) == 5
    assert b.steps == 11 and torch.equal(a.u_curr, b.u_curr) and torch.equal(a.u_prev, b.u_prev)
    if integrator == "bdf2":
        assert torch.equal(a.u_prev2, b.u_prev2) and torch.equal(a.u_prev3, b.u_prev3)
    with pytest.raises(ValueError):
        load_rollout(path, _FakeSolver(8, integrator))                 # other mesh size
    with pytest.raises(ValueError):
        load_rollout(path, _FakeSolver(7, "bdf2" if integrator == "be" else "be"))
    assert not list(tmp_path.glob("*.tmp.*"))                          # no temporary left behind


@pytest.mark.gpu
@pytest.mark.parametrize("batched", [False, True])
def test_resumed_rollout_equals_uninterrupted(tmp_path, batched):
    from simkit_gb300.batched import BatchedBESolver
    from simkit_gb300.beams import beam_batch, beam_small_steady
    from simkit_gb300.checkpoint import load_rollout, save_rollout
    from simkit_gb300.solver import BESolver
    if batched:
        specs = beam_batch(4, seed=1, nx_range=(4, 6), ny_range=(4, 5), nz_range=(8, 12))
        make = lambda: BatchedBESolver(specs)
    else:
        make = lambda: BESolver.from_spec(beam_small_steady(), coarse_refresh="step")
    a = make()
    for _ in range(5):
        a.step()
    save_rollout(tmp_path / "ck.npz", a, seed=3)
    for _ in range(4):
        a.step()
    b = make()
    assert load_rollout(tmp_path / "ck.npz", b) == 3 and b.steps == 5
    for _ in range(4):
        b.step()
    assert torch.equal(a.u_curr, b.u_curr) and torch.equal(a.u_prev, b.u_prev)


@pytest.mark.gpu
def test_network_checkpoint_restores_training_state(tmp_path):
    from simkit_gb300 import warmstart as ws
    from simkit_gb300.checkpoint import load_network, save_network
    a = ws.WarmStartMLP(seed=0)
    # a few Adam steps with synthetic gradients so the moments are non-zero
    for k in range(3):
        dWs = [torch.full_like(w, 1e-3 * (k + 1)) for w in a.W]
        dbs = [torch.full_like(b, -1e-3) for b in a.b]
        a.adam_step(dWs, dbs)
    save_network(tmp_path / "net.npz", a)
    b = ws.WarmStartMLP(seed=1)
    load_network(tmp_path / "net.npz", b)
    assert b.t == a.t
    for li in range(len(a.W)):
        for x, y in ((a.W, b.W), (a.b, b.b), (a.mW, b.mW), (a.vW, b.vW), (a.W16, b.W16), (a.WT16, b.WT16)):
            assert torch.equal(x[li], y[li]), li
    X = torch.randn(256, 64, generator=torch.Generator().manual_seed(2)).bfloat16().cuda()
    assert torch.equal(a.forward(X), b.forward(X))
