"""Parity on the benchmarked workload: the 786,432-tet beam (32 x 32 x 128 cubes, rest shape jittered by
U(-0.1, 0.1) cells, Young's modulus log-uniform [1e5, 1e7] per tet, seed 0), stepped by the
mixed-precision solver with the settings ``bench.py`` times (two-level grid PCG, Eisenstat-Walker forcing
capped at 0.3, coarse inverse rebuilt every 16 steps, Newton to a 1e-6 relative residual).

* Against simkit: the first two backward-Euler steps from rest, compared with
  ``golden/rollout_beam_32x32x128_first_steps.npz`` (simkit's energies, Hessians, line search and Newton;
  its spsolve replaced by a 1e-10 PCG because SuperLU does not finish on this mesh).
* Against the package's FP64 mode (FP64 element kernels, SpMV and dots, PCG forcing 1e-3): 30 steps.

Errors are stated two ways: positions relative to the largest rest coordinate (the stated 1e-5 bar) and
displacements relative to the largest displacement (the stricter measure: displacements are mm to cm).
"""

import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

FIXTURE = "rollout_beam_32x32x128_first_steps.npz"


def _bench_solver(spec, precision="mixed", variant=None):
    from simkit_gb300.solver import BESolver
    kw = dict(pcg_rtol=-0.3) if precision == "mixed" else dict(pcg_rtol=1e-3)
    s = BESolver.from_spec(spec, precision=precision, pcg_mode=3, coarse="auto", coarse_refresh=16, **kw)
    if variant is not None:
        s.params.pcg_variant = variant
    return s


@pytest.fixture(scope="module")
def c2_spec():
    from simkit_gb300.beams import beam_large_jittered
    return beam_large_jittered(seed=0)


# variant 13: the three-barrier two-level kernel the autotuner picked on a GB300; 18: its two-barrier form
@pytest.mark.parametrize("variant", [13, 18])
def test_c2_first_steps_match_simkit(c2_spec, variant):
    d = np.load(os.path.join(GOLDEN, FIXTURE))
    spec = c2_spec
    assert tuple(int(v) for v in d["dims"]) == spec.dims
    sample = d["sample"]
    s = _bench_solver(spec, variant=variant)
    X = spec.X[sample]
    scale = np.abs(spec.X).max()
    for k, step in enumerate(d["steps"]):
        while s.steps < int(step):
            info = s.step()
            assert info.converged, info
        u = s.displacement().reshape(-1, 3)[sample]
        u_ref = d["u"][k]
        pos = np.abs((X + u) - (X + u_ref)).max() / scale
        disp = np.abs(u - u_ref).max() / np.abs(u_ref).max()
        print(f"\nstep {int(step)}: positions rel err {pos:.2e}, displacement rel err {disp:.2e}, "
              f"newton {info.newton_iters} (simkit, exact solves: {int(d['iters'][k])})")
        assert pos < 2e-10     # measured 1.5e-11 (step 1), 3.5e-11 (step 2)
        assert disp < 1e-7     # measured 1.7e-8, 1.3e-8


def test_c2_mixed_matches_fp64_mode_over_30_steps(c2_spec):
    spec = c2_spec
    a = _bench_solver(spec, "mixed")
    b = _bench_solver(spec, "fp64")
    scale = np.abs(spec.X).max()
    worst_pos = worst_disp = 0.0
    for step in range(1, 31):
        ia, ib = a.step(), b.step()
        assert ia.converged and ib.converged, (step, ia, ib)
        ua, ub = a.displacement(), b.displacement()
        worst_pos = max(worst_pos, np.abs(ua - ub).max() / scale)
        worst_disp = max(worst_disp, np.abs(ua - ub).max() / np.abs(ub).max())
    print(f"\n30 steps, mixed vs FP64 mode: positions rel err {worst_pos:.2e}, displacement rel err {worst_disp:.2e}")
    assert worst_pos < 5e-8    # measured 1.0e-8
    assert worst_disp < 2e-7   # measured 3.2e-8
