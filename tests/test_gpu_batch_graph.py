"""The batched step with the Newton loop on the device (one CUDA graph launch per step: per-instance
decisions in control kernels, Newton iterations and line-search trials as conditional graph nodes)
against the host-driven batched step, which makes the same decisions with the same arithmetic on the
host: bitwise the same positions and the same per-instance records, for backward Euler and BDF2, with
the learned warm start's residual-judged choice, with contact planes, and when the PCG is starved."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _pair(specs, **kw):
    from simkit_gb300.batched import BatchedBESolver
    g = BatchedBESolver(specs, graph=True, **kw)
    h = BatchedBESolver(specs, graph=False, **kw)
    return g, h


def _same_records(ig, tg, ih, th):
    for a, b in zip(ig, ih):
        assert (a.newton_iters, a.pcg_iters, a.ls_trials, a.status, a.warm_used) == \
               (b.newton_iters, b.pcg_iters, b.ls_trials, b.status, b.warm_used)
        assert a.residual0 == b.residual0 and a.residual == b.residual
        assert a.min_alpha == b.min_alpha and a.energy == b.energy
    assert (tg.newton_iters, tg.pcg_iters, tg.ls_trials, tg.status) == \
           (th.newton_iters, th.pcg_iters, th.ls_trials, th.status)


@pytest.mark.parametrize("coarse", ["auto", None])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_graph_step_equals_host_driven_step(coarse, precision):
    from simkit_gb300.beams import beam_batch
    specs = beam_batch(12, seed=7, nx_range=(4, 10), ny_range=(4, 8), nz_range=(8, 24))
    g, h = _pair(specs, coarse=coarse, precision=precision)
    for _ in range(4):
        ig, tg = g.step()
        ih, th = h.step()
        assert tg.status == 0 and th.status == 0
        _same_records(ig, tg, ih, th)
        assert torch.equal(g.u_curr, h.u_curr)
    assert len(g._plans) == 3          # one graph per rotation of the three state buffers
    assert tg.launches > 0


def test_graph_step_with_a_coarse_refresh_period():
    """Per-instance coarse inverses rebuilt every second step: the graph path keeps one graph per state
    rotation and refresh decision (a period of 2 against 3 rotations meets all six) and takes bitwise
    the host-driven path's steps."""
    from simkit_gb300.beams import beam_batch
    specs = beam_batch(8, seed=3, nx_range=(4, 8), ny_range=(4, 6), nz_range=(8, 16))
    g, h = _pair(specs, coarse="auto", coarse_refresh=2)
    for _ in range(7):
        ig, tg = g.step()
        ih, th = h.step()
        assert tg.status == 0 and th.status == 0
        _same_records(ig, tg, ih, th)
        assert torch.equal(g.u_curr, h.u_curr)
    assert len(g._plans) == 6          # three rotations x (rebuild, reuse)


def test_graph_step_bdf2_with_contact_and_warm_start():
    from simkit_gb300.beams import beam_batch
    specs = beam_batch(6, seed=9, nx_range=(4, 8), ny_range=(4, 6), nz_range=(8, 16))
    floor = [(1.0e4, (0.0, -0.01, 0.0), (0.0, 1.0, 0.0))]
    g, h = _pair(specs, integrator="bdf2", contact_planes=floor)
    rng = np.random.default_rng(0)
    for k in range(5):
        warm = None
        if k >= 2:   # a perturbed prediction: the energy test keeps it for some instances only
            warm = g.u_curr + 1e-4 * torch.from_numpy(rng.standard_normal(g.u_curr.numel())).cuda()
        ig, tg = g.step(u_warm=warm)
        ih, th = h.step(u_warm=warm)
        _same_records(ig, tg, ih, th)
        assert torch.equal(g.u_curr, h.u_curr)
    assert len(g._plans) == 5          # BDF2 rotates five buffers (steps 0-1 plain, 2-4 with the warm start)


def test_graph_reports_failures_like_the_host_loop():
    """A one-iteration PCG cap: every instance ends not converged after max_newton iterations, with
    the same records on both paths; parameters changed afterwards re-record the graphs."""
    from simkit_gb300 import _lib
    from simkit_gb300.beams import beam_batch
    specs = beam_batch(5, seed=4, nx_range=(4, 6), ny_range=(4, 5), nz_range=(8, 12))
    g, h = _pair(specs, pcg_max_iter=1, max_newton=3, coarse=None)
    ig, tg = g.step()
    ih, th = h.step()
    _same_records(ig, tg, ih, th)
    assert all(i.status == _lib.SKG_ERR_NOT_CONVERGED and i.newton_iters == 3 for i in ig)
    assert tg.status == _lib.SKG_ERR_NOT_CONVERGED
    for s in (g, h):
        s.params.pcg_max_iter = 4000
        s.params.max_newton = 20
    ig, tg = g.step()
    ih, th = h.step()
    _same_records(ig, tg, ih, th)
    assert tg.status == 0
    assert torch.equal(g.u_curr, h.u_curr)


def test_real_distribution_beams_match_oracle():
    """Beams drawn from the benchmarked 512-beam batch itself (seed 0: the smallest, the median and the
    90th-percentile instance, 1,200 to 36,288 tets, each with its own E, nu and gravity direction),
    stepped in one batch with the default settings (mixed precision, two-level cluster PCG, device
    Newton loop), against the FP64 oracle's first two steps."""
    from oracle import rollout
    from simkit_gb300.batched import BatchedBESolver
    from simkit_gb300.beams import beam_batch
    every = beam_batch(512, seed=0)
    sizes = np.array([s.n_tets for s in every])
    order = np.argsort(sizes, kind="stable")
    specs = [every[int(order[0])], every[int(order[len(order) // 2])], every[int(order[int(0.9 * len(order))])]]
    b = BatchedBESolver(specs)
    refs = [rollout.from_spec(sp) for sp in specs]
    states = [(r.x_rest.copy(), r.x_rest.copy()) for r in refs]
    worst_pos = worst_disp = 0.0
    for _ in range(2):
        infos, total = b.step()
        assert total.status == 0, total
        for i, sp in enumerate(specs):
            xc, xp = states[i]
            xn, info = refs[i].step(xc, xp)
            assert info.converged
            states[i] = (xn, xc)
            X = sp.X.reshape(-1)
            u, u_ref = b.displacement(i), xn.ravel() - X
            worst_pos = max(worst_pos, np.abs(u - u_ref).max() / np.abs(X).max())
            worst_disp = max(worst_disp, np.abs(u - u_ref).max() / np.abs(u_ref).max())
    print(f"\nreal-distribution beams vs oracle: positions rel err {worst_pos:.2e}, displacement rel err {worst_disp:.2e}")
    assert worst_pos < 1e-7
    assert worst_disp < 5e-6
