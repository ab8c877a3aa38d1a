"""The allocation-free PCG entry point against the allocating one.

skg_pcg_bsr64_noalloc serves callers that cannot allocate device memory
while they solve (a real-time loop that must not stall on cudaMalloc, or a
host program that owns all device buffers and passes only inputs and
outputs); its scratch is a fixed array inside the library.  These checks call
both entry points through the C ABI on the same system and compare the
solutions, twice in a row, so a stale scratch array from the first call would
show up in the second.  This file runs last so that a failure here leaves
every other test already run.
"""

import ctypes

import numpy as np
import pytest
import scipy.sparse as sps
import torch

pytestmark = pytest.mark.gpu

RTOL_SOLVE = 1e-12      # PCG stopping tolerance of both calls
RTOL_COMPARE = 1e-9     # agreement required between the two entry points


def _entry_major(A):
    """Symmetric scalar matrix (3m x 3m) -> block rows in the library's layout."""
    Ab = sps.bsr_matrix(A, blocksize=(3, 3))
    Ab.sort_indices()
    nbr = A.shape[0] // 3
    rowptr = Ab.indptr.astype(np.int64)
    cols = Ab.indices.astype(np.int64)
    rows = np.repeat(np.arange(nbr), np.diff(rowptr))
    K = np.diff(rowptr)
    k = np.arange(cols.size) - rowptr[rows]
    val = np.empty(9 * cols.size)
    for m in range(9):
        val[9 * rowptr[rows] + m * K[rows] + k] = Ab.data[:, m // 3, m % 3]
    return nbr, rowptr.astype(np.int32), cols.astype(np.int32), val


def _system(seed):
    """Stiffness of a small pinned-free beam plus M/h^2: symmetric positive definite."""
    from simkit_gb300.beams import make_beam
    from oracle import fem, snh
    b = make_beam(10, 4, 4, ym=1e6, pr=0.45, jitter=0.1, seed=seed)
    J = fem.deformation_jacobian(b.X, b.T)
    x = b.X + 1e-3 * np.random.default_rng(seed).standard_normal(b.X.shape)
    K = snh.hessian_x(x, J, b.mu, b.lam, fem.tet_volumes(b.X, b.T))
    m = np.repeat(fem.lumped_mass(b.X, b.T, 1000.0), 3)
    return (K + sps.diags(m * 3600.0)).tocsr()


def _solve_both(lib, A, b):
    nbr, rowptr, col, val = _entry_major(A)
    dev = lambda a: torch.from_numpy(a).cuda()
    rp_d, col_d, val_d, b_d = dev(rowptr), dev(col), dev(val), dev(b)
    x_ref = torch.empty(3 * nbr, dtype=torch.float64, device="cuda")
    x_na = torch.full((3 * nbr,), float("nan"), dtype=torch.float64, device="cuda")
    ws = torch.empty(int(lib.skg_pcg_workspace_size(nbr)), dtype=torch.uint8, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    it_ref, it_na = ctypes.c_int32(), ctypes.c_int32()
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert lib.skg_pcg_bsr64(nbr, p(rp_d), p(col_d), p(val_d), p(b_d), p(x_ref), RTOL_SOLVE, 20000,
                             ctypes.byref(it_ref), p(ws), stream) == 0
    assert lib.skg_pcg_bsr64_noalloc(nbr, p(rp_d), p(col_d), p(val_d), p(b_d), p(x_na), RTOL_SOLVE, 20000,
                                     ctypes.byref(it_na), stream) == 0
    torch.cuda.synchronize()
    return x_ref.cpu().numpy(), x_na.cpu().numpy(), it_ref.value, it_na.value


def test_noalloc_pcg_matches_allocating_entry_point_twice():
    from simkit_gb300 import _lib
    lib = _lib.load()
    A = _system(1)
    assert A.shape[0] // 3 <= lib.skg_pcg_noalloc_max_rows()
    rng = np.random.default_rng(0)
    for call in range(2):
        b = rng.standard_normal(A.shape[0])
        x_ref, x_na, it_ref, it_na = _solve_both(lib, A, b)
        assert np.all(np.isfinite(x_na)), call
        err = np.linalg.norm(x_na - x_ref) / np.linalg.norm(x_ref)
        assert err <= RTOL_COMPARE, (call, err)
        assert it_na == it_ref
        # and the solution solves the system
        assert np.linalg.norm(A @ x_na - b) <= 1e-9 * np.linalg.norm(b)


def test_noalloc_pcg_rejects_systems_beyond_its_capacity():
    from simkit_gb300 import _lib
    lib = _lib.load()
    cap = int(lib.skg_pcg_noalloc_max_rows())
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(dummy.data_ptr())
    st = lib.skg_pcg_bsr64_noalloc(cap + 1, p, p, p, p, p, 1e-8, 10, None, None)
    assert st == _lib.SKG_ERR_CAPACITY
    assert "capacity" in _lib.last_error()


def _block_tridiagonal(nbr, seed):
    """A symmetric positive definite block-tridiagonal system with nbr 3x3 block rows (diagonally
    dominant blocks), to fill the fixed scratch to its capacity."""
    rng = np.random.default_rng(seed)
    n = 3 * nbr
    # the coupling of block row i to block row i + 1: every scalar offset 1..5 that lands there
    rows, cols, vals = [], [], []
    for d in range(1, 6):
        i = np.arange(n - d)
        keep = (i + d) // 3 == i // 3 + 1
        rows.append(i[keep]); cols.append(i[keep] + d); vals.append(rng.uniform(-1.0, 1.0, keep.sum()))
    band = sps.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    A = band + band.T
    # a dense symmetric 3x3 diagonal block per row, dominant over the row's off-diagonal sum
    Dd = rng.uniform(-0.5, 0.5, size=(nbr, 3, 3))
    Dd = Dd + Dd.transpose(0, 2, 1)
    rows = np.repeat(np.arange(nbr) * 3, 9) + np.tile(np.repeat(np.arange(3), 3), nbr)
    cols = np.repeat(np.arange(nbr) * 3, 9) + np.tile(np.tile(np.arange(3), 3), nbr)
    A = A + sps.csr_matrix((Dd.reshape(-1), (rows, cols)), shape=(n, n))
    rowsum = np.asarray(abs(A).sum(axis=1)).ravel()
    return (A + sps.diags(rowsum + 1.0)).tocsr()


def test_noalloc_pcg_at_full_capacity_matches_allocating_entry_point():
    """A system of exactly skg_pcg_noalloc_max_rows() block rows fits the fixed scratch and gives the
    allocating entry point's answer (twice, so the second call starts from the first one's scratch)."""
    from simkit_gb300 import _lib
    lib = _lib.load()
    cap = int(lib.skg_pcg_noalloc_max_rows())
    A = _block_tridiagonal(cap, 5)
    assert A.shape[0] // 3 == cap
    rng = np.random.default_rng(1)
    for call in range(2):
        b = rng.standard_normal(A.shape[0])
        x_ref, x_na, it_ref, it_na = _solve_both(lib, A, b)
        err = np.linalg.norm(x_na - x_ref) / np.linalg.norm(x_ref)
        assert err <= RTOL_COMPARE, (call, err)
        assert it_na == it_ref
        assert np.linalg.norm(A @ x_na - b) <= 1e-9 * np.linalg.norm(b)
