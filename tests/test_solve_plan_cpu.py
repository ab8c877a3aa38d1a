"""The block plan behind ``solve_sparse`` for scipy matrices (host only): the scatter of scalar CSR
values into the PCG's entry-major 3x3-block values equals a loop over the dense matrix and the stored
entries, with diagonal blocks added where the matrix has none (zero blocks included: the PCG needs
every diagonal block), rows padded to a multiple of 3 with the identity
and repeated entries of a non-canonical CSR summed; the plan is reused for the same pattern only."""

import numpy as np
import scipy.sparse as sps

from simkit_gb300.api import _BlockPlan, _diagonal_of


def _reference_values(A):
    """Block pattern and entry-major block values by loops over the stored entries: a block (I, J)
    exists where A stores an entry or I == J; rows past n get the identity."""
    n = A.shape[0]
    N = n + (-n) % 3
    nbr = N // 3
    D = np.zeros((N, N))
    D[:n, :n] = A.toarray()
    D[np.arange(n, N), np.arange(n, N)] = 1.0
    Ac = A.tocoo()
    blocks = {(i, i) for i in range(nbr)} | {(int(r) // 3, int(c) // 3) for r, c in zip(Ac.row, Ac.col)}
    rowptr = [0]
    col = []
    for I in range(nbr):
        cs = sorted(J for (Ii, J) in blocks if Ii == I)
        col += cs
        rowptr.append(len(col))
    rowptr = np.array(rowptr)
    val = np.zeros(9 * len(col))
    for I in range(nbr):
        K = rowptr[I + 1] - rowptr[I]
        for k in range(K):
            J = col[rowptr[I] + k]
            for m in range(9):
                val[9 * rowptr[I] + m * K + k] = D[3 * I + m // 3, 3 * J + m % 3]
    return rowptr, np.array(col), val


def test_plan_matches_scipy_bsr_values():
    rng = np.random.default_rng(0)
    for n in (30, 31, 32, 99):
        A = sps.random(n, n, density=0.08, random_state=int(rng.integers(1 << 30)), format="csr")
        A = (A + A.T + sps.identity(n) * 0.0).tocsr()
        A.sort_indices()
        plan = _BlockPlan(A.indptr, A.indices, n)
        rowptr, col, val = _reference_values(A)
        assert np.array_equal(plan.rowptr, rowptr) and np.array_equal(plan.col, col)
        assert np.array_equal(plan.values(A.data), val)
        assert plan.N == n + (-n) % 3


def test_plan_sums_repeated_entries_and_matches_only_its_pattern():
    rows = np.array([0, 0, 1, 2, 2, 2])
    cols = np.array([0, 0, 1, 2, 0, 2])
    data = np.array([1.0, 2.0, 3.0, 4.0, 5.0, 6.0])
    A = sps.csr_matrix((data, cols, np.array([0, 2, 3, 6])), shape=(3, 3))   # not canonical: (0,0), (2,2) twice
    plan = _BlockPlan(A.indptr, A.indices, 3)
    val = plan.values(A.data)
    assert val[0] == 3.0 and val[8] == 10.0 and val[6] == 5.0    # entry-major 3x3 of the one block
    assert plan.matches(A)
    B = sps.csr_matrix(np.eye(3))
    assert not plan.matches(B)


def test_diagonal_detection():
    d = np.arange(1.0, 7.0)
    assert np.array_equal(_diagonal_of(sps.diags(d), 6), d)
    assert np.array_equal(_diagonal_of(np.diag(d), 6), d)
    assert _diagonal_of(sps.diags(d) + sps.eye(6, k=1), 6) is None
    assert _diagonal_of(sps.diags(d), 5) is None
