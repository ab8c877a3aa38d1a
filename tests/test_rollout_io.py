"""Trajectory caches in simkit's compute_with_cache_check format."""

import os

import numpy as np
import pytest

from simkit_gb300.rollout_io import compute_with_cache_check

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_reads_a_cache_written_by_simkit(tmp_path):
    """A file simkit wrote (array, int, one-element array, array) reads back with simkit's
    conversions: scalars and one-element arrays become Python scalars."""
    calls = []
    out = compute_with_cache_check(lambda: calls.append(1), os.path.join(GOLDEN, "cache_reference.npz"))
    assert not calls
    traj, n, s, a = out
    assert traj.shape == (3, 5, 3) and isinstance(n, int) and n == 7
    assert isinstance(s, float) and s == 2.5
    assert np.array_equal(a, np.arange(4))


def test_writes_simkit_keys_and_reads_back(tmp_path):
    path = str(tmp_path / "traj.npz")
    rng = np.random.default_rng(0)
    x = rng.standard_normal((4, 6, 3))
    out = compute_with_cache_check(lambda: (x, np.array([3, 4])), path)
    assert np.load(path).files == ["v0", "v1"]
    again = compute_with_cache_check(lambda: pytest.fail("recomputed"), path)
    assert np.array_equal(again[0], x) and np.array_equal(again[1], [3, 4])
    single = compute_with_cache_check(lambda: x, str(tmp_path / "one.npz"), read_cache=False)
    assert isinstance(single, tuple) and np.array_equal(single[0], x)


@pytest.mark.gpu
def test_cached_device_rollout(tmp_path):
    from simkit_gb300.beams import make_beam
    from simkit_gb300.rollout_io import cached_rollout
    from simkit_gb300.solver import BESolver
    spec = make_beam(4, 2, 2, ym=3e5, pr=0.4)
    s = BESolver.from_spec(spec)
    path = str(tmp_path / "beam.npz")
    traj, iters, res = cached_rollout(s, 5, path)
    assert traj.shape == (6, spec.n_verts, 3) and np.array_equal(traj[0], spec.X)
    assert np.all(res < 1e-6) and np.all(iters >= 1)
    assert np.allclose(traj[-1], spec.X + s.displacement().reshape(-1, 3))
    traj2, iters2, res2 = cached_rollout(s, 5, path)       # read from the file, no stepping
    assert s.steps == 5 and np.array_equal(traj2, traj) and np.array_equal(iters2, iters)
