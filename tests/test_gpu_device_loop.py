"""The single-mesh step with the Newton loop on the device (``skg_be_plan_*``: one CUDA graph launch
per step, the decisions in control kernels, Newton iterations and line-search trials as conditional
graph nodes, the PCG reading its forcing term from device memory) against the host loop of
``skg_be_step``, which makes the same decisions with the same arithmetic on the host: bitwise the same
displacements and the same step records, on a jittered beam with E log-uniform over [1e5, 1e7] above
the cluster size (the grid PCG forms), one- and two-level, FP64 and mixed, with the coarse inverse
rebuilt every second step, and when the PCG is starved."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spec():
    from simkit_gb300.beams import beam_large_jittered
    return beam_large_jittered(nx=96, ny=16, nz=16, seed=4)   # 28,033 vertices, 147,456 tets


def _pair(spec, **kw):
    from simkit_gb300.solver import BESolver
    return BESolver.from_spec(spec, device_loop=True, **kw), BESolver.from_spec(spec, device_loop=False, **kw)


def _same(a, b):
    assert (a.newton_iters, a.pcg_iters, a.ls_trials, a.status) == (b.newton_iters, b.pcg_iters, b.ls_trials, b.status)
    assert a.residual0 == b.residual0 and a.residual == b.residual
    assert a.min_alpha == b.min_alpha and a.energy == b.energy


@pytest.mark.parametrize("coarse", ["auto", None])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_device_loop_equals_host_loop(coarse, precision):
    from simkit_gb300 import _lib
    spec = _spec()
    g, h = _pair(spec, coarse=coarse, precision=precision, coarse_refresh=2, pcg_rtol=-0.3)
    assert _lib.load().skg_be_plan_eligible(g.mesh.c, g.params) == 1
    for _ in range(4):
        ig, ih = g.step(), h.step()
        assert ig.converged and ih.converged, (ig, ih)
        _same(ig, ih)
        assert np.array_equal(g.u_curr.cpu().numpy(), h.u_curr.cpu().numpy())
    assert len(g._plans) >= 3 and len(h._plans) == 0     # three state rotations, two refresh decisions


def test_device_loop_reports_a_starved_pcg_like_the_host_loop():
    from simkit_gb300 import _lib
    spec = _spec()
    g, h = _pair(spec, coarse=None, pcg_max_iter=1, max_newton=3, pcg_rtol=1e-8)
    ig, ih = g.step(), h.step()
    assert ig.status == _lib.SKG_ERR_NOT_CONVERGED and ig.newton_iters == 3
    _same(ig, ih)
    assert np.array_equal(g.u_curr.cpu().numpy(), h.u_curr.cpu().numpy())


def test_host_loop_where_the_device_loop_does_not_apply():
    """Profiled steps, simkit's stop rule and the cluster PCG of small meshes take the host loop."""
    from simkit_gb300 import _lib
    from simkit_gb300.beams import make_beam
    from simkit_gb300.solver import BESolver
    lib = _lib.load()
    g = BESolver.from_spec(_spec(), device_loop=True)
    g.params.profile = 1
    assert lib.skg_be_plan_eligible(g.mesh.c, g.params) == 0
    info = g.step()
    assert info.converged and info.t_pcg_ms > 0.0 and len(g._plans) == 0
    g.params.profile = 0
    g.params.stop_rule = 1
    assert lib.skg_be_plan_eligible(g.mesh.c, g.params) == 0
    small = BESolver.from_spec(make_beam(8, 3, 3), device_loop=True)
    assert lib.skg_be_plan_eligible(small.mesh.c, small.params) == 0
    assert small.step().converged and len(small._plans) == 0


def test_device_loop_bdf2_with_contact_equals_host_loop():
    """BDF2 (five displacement levels rotate, five graphs) with a floor contact plane."""
    spec = _spec()
    floor = [(1.0e4, (0.0, -0.01, 0.0), (0.0, 1.0, 0.0))]
    g, h = _pair(spec, integrator="bdf2", contact_planes=floor, coarse_refresh=3)
    for _ in range(6):
        ig, ih = g.step(), h.step()
        assert ig.converged and ih.converged, (ig, ih)
        _same(ig, ih)
        assert np.array_equal(g.u_curr.cpu().numpy(), h.u_curr.cpu().numpy())
    assert len(g._plans) >= 5


def test_prepare_plans_records_every_rotation_up_front():
    """Three state rotations x (rebuild, reuse) recorded before the first step; stepping adds none."""
    spec = _spec()
    g, h = _pair(spec, coarse_refresh=2)
    assert g.prepare_plans() == 6
    for _ in range(4):
        ig, ih = g.step(), h.step()
        _same(ig, ih)
    assert len(g._plans) == 6
    assert np.array_equal(g.u_curr.cpu().numpy(), h.u_curr.cpu().numpy())
    g.params.tol = 1e-7            # a parameter change re-records on the next step
    g.step()
    assert len(g._plans) == 1
