"""Failure detection on the GPU, with every failure made on the host or by a wait that nothing ends.

* Bounded waits: the grid barrier of the grid-persistent PCG forms and the mbarrier wait of the cluster
  PCG run on a condition nothing meets (``skg_wait_selftest``) and return SKG_ERR_TIMEOUT after a short
  poll limit; the context stays usable (a solve runs right after).
* PCG non-convergence: an iteration cap too small for the tolerance gives SKG_ERR_NOT_CONVERGED with
  the reached residual in the message (simkit's newton/spsolve path has no such status), and a
  Newton step with a one-iteration PCG reports not converged instead of returning a silent result.
* Bad meshes made on the host: a tet with a vertex index outside the mesh (the setup kernel does not
  read it), a zero-volume tet and a tet inverted at rest are refused before any solve.
* Inverted elements in the state (a vertex pushed through its neighbours on the host): the step
  recovers like the FP64 oracle does.
"""

import ctypes

import numpy as np
import pytest
import scipy.sparse as sps
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from simkit_gb300 import _lib
    return _lib.load()


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("kind", [0, 1])
def test_stuck_wait_returns_timeout_status(lib, kind):
    from simkit_gb300 import _lib
    ws = torch.empty(int(lib.skg_wait_selftest_workspace_size()), dtype=torch.uint8, device="cuda")
    st = ctypes.c_int32(12345)
    limit = 1 << 16 if kind == 0 else 1 << 10
    assert lib.skg_wait_selftest(kind, limit, ctypes.byref(st), _p(ws), None) == 0
    assert st.value == _lib.SKG_ERR_TIMEOUT
    # the context is still usable: a solve right after runs and converges
    A = sps.diags(np.linspace(1.0, 3.0, 30)).tocsr()
    x = _solve(lib, A, np.ones(30), 1e-10, 200)[0]
    assert np.allclose(A @ x, 1.0, atol=1e-8)


def test_wait_selftest_rejects_bad_arguments(lib):
    from simkit_gb300 import _lib
    ws = torch.empty(256, dtype=torch.uint8, device="cuda")
    st = ctypes.c_int32()
    assert lib.skg_wait_selftest(2, 10, ctypes.byref(st), _p(ws), None) == _lib.SKG_ERR_ARG
    assert lib.skg_wait_selftest(0, 0, ctypes.byref(st), _p(ws), None) == _lib.SKG_ERR_ARG


def _solve(lib, A, b, rtol, max_iter):
    """skg_pcg_bsr64 on a scalar SPD matrix whose size is a multiple of 3; returns (x, status, iters)."""
    Ab = sps.bsr_matrix(A, blocksize=(3, 3))
    Ab.sort_indices()
    nbr = A.shape[0] // 3
    rowptr = Ab.indptr.astype(np.int64)
    rows = np.repeat(np.arange(nbr), np.diff(rowptr))
    K = np.diff(rowptr)
    k = np.arange(Ab.indices.size) - rowptr[rows]
    val = np.empty(9 * Ab.indices.size)
    for m in range(9):
        val[9 * rowptr[rows] + m * K[rows] + k] = Ab.data[:, m // 3, m % 3]
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    rp, col, v, bd = d(rowptr.astype(np.int32)), d(Ab.indices.astype(np.int32)), d(val), d(b.astype(np.float64))
    x = torch.empty(3 * nbr, dtype=torch.float64, device="cuda")
    ws = torch.empty(int(lib.skg_pcg_workspace_size(nbr)), dtype=torch.uint8, device="cuda")
    it = ctypes.c_int32()
    st = lib.skg_pcg_bsr64(nbr, _p(rp), _p(col), _p(v), _p(bd), _p(x), rtol, max_iter, ctypes.byref(it), _p(ws), None)
    return x.cpu().numpy(), st, it.value


def test_pcg_iteration_cap_reports_not_converged(lib):
    from simkit_gb300 import _lib
    n = 3 * 200
    A = sps.diags([-np.ones(n - 1), 2.0 * np.ones(n) + 1e-3, -np.ones(n - 1)], [-1, 0, 1]).tocsr()
    b = np.random.default_rng(0).standard_normal(n)
    _, st, it = _solve(lib, A, b, 1e-12, 3)
    assert st == _lib.SKG_ERR_NOT_CONVERGED and it == 3
    assert "relative residual" in _lib.last_error()
    x, st, _ = _solve(lib, A, b, 1e-12, 5000)
    assert st == 0 and np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_newton_with_starved_pcg_reports_not_converged(precision):
    from simkit_gb300 import _lib
    from simkit_gb300.beams import make_beam
    from simkit_gb300.solver import BESolver
    spec = make_beam(8, 3, 3, ym=1e6, pr=0.45)
    s = BESolver.from_spec(spec, precision=precision, pcg_max_iter=1, max_newton=2, coarse=None, pcg_rtol=1e-8)
    info = s.step()
    assert info.status == _lib.SKG_ERR_NOT_CONVERGED
    assert info.newton_iters == 2 and info.residual > 1e-6


def test_tet_setup_skips_out_of_range_vertex(lib):
    """The C ABI's setup kernel does not read a vertex index outside [0, n): that tet gets NaN."""
    from simkit_gb300.beams import beam_mesh
    X, T = beam_mesh(2, 1, 1)
    T = T.astype(np.int32).copy()
    T[3, 2] = X.shape[0]            # one past the last vertex
    T[5, 0] = -7
    Xd = torch.from_numpy(X.reshape(-1)).cuda()
    Td = torch.from_numpy(T).cuda()
    t = T.shape[0]
    dinv = torch.empty(9 * t, dtype=torch.float64, device="cuda")
    vol = torch.empty(t, dtype=torch.float64, device="cuda")
    assert lib.skg_tet_setup(_p(Xd), _p(Td), X.shape[0], t, _p(dinv), _p(vol), None) == 0
    v = vol.cpu().numpy()
    assert np.isnan(v[3]) and np.isnan(v[5])
    assert np.all(v[[0, 1, 2, 4] + list(range(6, t))] > 0)


def test_degenerate_and_inverted_rest_tets_are_refused():
    from simkit_gb300.beams import make_beam
    from simkit_gb300.mesh import TetMesh
    from simkit_gb300.solver import BESolver
    spec = make_beam(3, 2, 2)
    flat = spec.X.copy()
    T = spec.T.copy()
    flat[T[4, 3]] = flat[T[4, 0]]      # two corners of tet 4 coincide: zero volume
    with pytest.raises(ValueError, match="degenerate"):
        TetMesh(flat, T, spec.mu, spec.lam)
    Ti = T.copy()
    Ti[7, [1, 2]] = Ti[7, [2, 1]]      # tet 7 with its orientation reversed
    with pytest.raises(ValueError, match="inverted at rest"):
        BESolver(spec.X, Ti, spec.mu, spec.lam, pinned=spec.pinned)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("mixed", 2e-4)])
def test_step_recovers_from_inverted_elements_like_the_oracle(precision, tol):
    """Two tets inverted in the initial state (a tip vertex pushed through its neighbours on the host):
    one step agrees with the FP64 oracle's step from the same state (which needs 7 Newton iterations).
    Measured on a GB300: 1.3e-14 (FP64) and, in mixed precision (FP32 Hessians, the same 1e-6 relative
    residual stop), 2.6e-5 with the Eisenstat-Walker exponent 2 and 1.04e-4 with 1.25 of the
    displacement, which here is 1.5 cells: two solutions that each meet the stop rule on this
    ill-conditioned state differ by that much."""
    from oracle import rollout
    from simkit_gb300.beams import make_beam
    from simkit_gb300.solver import BESolver
    spec = make_beam(6, 2, 2, ym=2e5, pr=0.45)
    ref = rollout.from_spec(spec)
    X = spec.X
    v = np.nonzero(np.isclose(X[:, 0], X[:, 0].max()))[0][-1]
    x = X.copy()
    x[v] += np.array([-1.5, 0.3, 0.0]) * 0.025
    F = (ref.J @ x.reshape(-1, 1)).reshape(-1, 3, 3)
    assert (np.linalg.det(F) < 0).sum() == 2
    xn, info_ref = ref.step(x.reshape(-1, 1), x.reshape(-1, 1))
    assert info_ref.converged
    kw = dict(pcg_rtol=1e-10) if precision == "fp64" else {}
    s = BESolver.from_spec(spec, precision=precision, coarse=None, **kw)
    u = (x - X).reshape(-1)
    s.set_state(u, u)
    info = s.step()
    assert info.converged, info
    got = X.reshape(-1) + s.displacement()
    err = np.abs(got - xn.ravel()).max() / np.abs(xn - X.reshape(-1, 1)).max()
    print(f"\n{precision}: displacement rel err {err:.2e}, newton {info.newton_iters} (oracle {info_ref.iters})")
    assert err < tol
