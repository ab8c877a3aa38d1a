"""Host-side checks of the two-level preconditioner (no GPU).

- ``coarse_aggregates`` data: the mode vectors, masks and coarse block pattern
  give, through the per-block formula the Galerkin kernel evaluates
  (C = [[A', -A' S_w], [S_v A', -S_v A' S_w]]), exactly P^T A P with P built
  column by column from the rigid modes;
- the blocked Gauss-Jordan schedule of the inversion kernel (32-wide pivot
  blocks, work units of 32 rows x 256 columns, panels read from the copies the
  previous step wrote) reproduces the inverse of an SPD matrix;
- the additive two-level preconditioner built from these pieces cuts the
  CG iterations of a stiff beam against block Jacobi.
"""

import numpy as np
import pytest
import scipy.sparse as sps

from simkit_gb300.mesh import coarse_aggregates
from simkit_gb300.beams import make_beam
from oracle import fem, snh

KB, KC = 32, 256


def _system(nx=12, ny=4, nz=4, ym=1e6, seed=0):
    sp = make_beam(nx, ny, nz, ym=ym, pr=0.45, jitter=0.1, seed=seed)
    J = fem.deformation_jacobian(sp.X, sp.T)
    vol = fem.tet_volumes(sp.X, sp.T)
    K = snh.hessian_x(sp.X.reshape(-1, 1), J, sp.mu, sp.lam, vol)
    m = fem.lumped_mass(sp.X, sp.T, 1000.0)
    H = (K + sps.diags(np.repeat(m, 3)) * 3600.0).tocsr()
    n = sp.X.shape[0]
    pin = np.zeros(3 * n, bool)
    pin[(3 * sp.pinned[:, None] + np.arange(3)).ravel()] = True
    # pinned rows / columns as the assembly writes them: identity on the diagonal
    D = sps.diags((~pin).astype(float))
    H = (D @ H @ D + sps.diags(pin.astype(float))).tocsr()
    return sp, H, pin


def _bsr_pattern(H, n):
    B = sps.bsr_matrix(H, blocksize=(3, 3))
    B.sort_indices()
    return B.indptr.astype(np.int32), B.indices.astype(np.int32), B.data


def _explicit_P(mode, n, n_agg):
    bits = mode[:, 3].view(np.uint32)
    agg = (bits & 0x1FFFFFFF).astype(np.int64)
    mask = bits >> 29
    d = mode[:, :3].astype(np.float64)
    P = np.zeros((3 * n, 6 * n_agg))
    for v in range(n):
        a = agg[v]
        S = np.array([[0, -d[v, 2], d[v, 1]], [d[v, 2], 0, -d[v, 0]], [-d[v, 1], d[v, 0], 0]])
        Pv = np.hstack([np.eye(3), -S])
        for c in range(3):
            if (mask[v] >> c) & 1:
                P[3 * v + c, 6 * a:6 * a + 6] = Pv[c]
    return P


def _galerkin_blocks(cd, rowptr, col, blocks, n):
    """The Galerkin kernel's arithmetic, block by block (no diagonal shift)."""
    n_agg = cd["n_agg"]
    mode = cd["mode"]
    bits = mode[:, 3].view(np.uint32)
    mask = bits >> 29
    d = mode[:, :3].astype(np.float64)
    row = np.repeat(np.arange(n), np.diff(rowptr))
    Ac = np.zeros((6 * n_agg, 6 * n_agg))

    def skew(x):
        return np.array([[0, -x[2], x[1]], [x[2], 0, -x[0]], [-x[1], x[0], 0]])

    for cb in range(cd["cb_ptr"].size - 1):
        ra, ca = cd["cb_rc"][2 * cb], cd["cb_rc"][2 * cb + 1]
        acc = np.zeros((6, 6))
        for k in range(cd["cb_ptr"][cb], cd["cb_ptr"][cb + 1]):
            s = cd["cb_slot"][k]
            v, w = row[s], col[s]
            fv = np.array([(mask[v] >> i) & 1 for i in range(3)], float)
            fw = np.array([(mask[w] >> i) & 1 for i in range(3)], float)
            a = blocks[s] * fv[:, None] * fw[None, :]
            Sv, Sw = skew(d[v]), skew(d[w])
            B = a @ Sw
            acc[:3, :3] += a
            acc[:3, 3:] -= B
            acc[3:, :3] += Sv @ a
            acc[3:, 3:] -= Sv @ B
        Ac[6 * ra:6 * ra + 6, 6 * ca:6 * ca + 6] = acc
    return Ac


def test_galerkin_formula_matches_ptap():
    sp, H, pin = _system()
    n = sp.X.shape[0]
    rowptr, col, blocks = _bsr_pattern(H, n)
    cd = coarse_aggregates(sp.X, ~pin, rowptr, col, box=4)
    assert cd["n_agg"] > 4
    # every fine slot lands in exactly one coarse block, grouped contiguously
    assert np.array_equal(np.sort(cd["cb_slot"]), np.arange(col.size))
    P = _explicit_P(cd["mode"], n, cd["n_agg"])
    ref = P.T @ H.toarray() @ P
    Ac = _galerkin_blocks(cd, rowptr, col, blocks, n)
    assert np.abs(Ac - ref).max() <= 1e-9 * np.abs(ref).max()
    # pinned DOFs carry no coarse mode
    assert np.all(P[pin] == 0.0)


def _gj_schedule(Min):
    """The inversion kernel's schedule in numpy (FP64): the symmetric sweep
    (M_KK <- -Pinv, M_KJ <- Pinv R_J, M_IK <- C_I Pinv, M_IJ <- M_IJ - C_I Pinv R_J with C = R^T)
    over the upper triangle of 32-row blocks, row panels written by the previous step, then the
    mirror pass that fills the lower triangle and flips the sign."""
    M = Min.copy()
    np_ = M.shape[0]
    nbk, ncu = np_ // KB, (np_ + KC - 1) // KC
    M[np.tril_indices(np_, -KB)] = np.nan     # below the diagonal blocks: never read
    for ib in range(nbk):
        M[ib * KB:(ib + 1) * KB, :ib * KB] = np.nan
    rowp = np.zeros((2, KB, np_))
    rowp[0] = Min[:KB, :]
    for kb in range(nbk):
        Rw = rowp[kb & 1].copy()
        K0, K1 = kb * KB, kb * KB + KB
        piv = np.linalg.inv(Rw[:, K0:K1])
        for ib in range(nbk):
            I0 = ib * KB
            for cu in range(I0 // KC, ncu):
                vt = piv if ib == kb else Rw[:, I0:I0 + KB].T @ piv   # V = C_I Pinv, C_I = R[:, I]^T
                for j in range(max(cu * KC, I0), min(np_, cu * KC + KC)):
                    if K0 <= j < K1:
                        a = -piv[:, j - K0] if ib == kb else vt[:, j - K0]
                    elif ib == kb:
                        a = vt @ Rw[:, j]
                    else:
                        a = M[I0:I0 + KB, j] - vt @ Rw[:, j]
                    M[I0:I0 + KB, j] = a
                    if kb + 1 < nbk:
                        if ib == kb + 1:
                            rowp[(kb + 1) & 1][:, j] = a
                        elif K1 <= j < K1 + KB and ib < kb + 1:
                            rowp[(kb + 1) & 1][j - K1, I0:I0 + KB] = a
    out = np.empty_like(M)
    for ib in range(nbk):
        for jb in range(ib, nbk):
            t = M[ib * KB:(ib + 1) * KB, jb * KB:(jb + 1) * KB]
            out[ib * KB:(ib + 1) * KB, jb * KB:(jb + 1) * KB] = -t
            if jb > ib:
                out[jb * KB:(jb + 1) * KB, ib * KB:(ib + 1) * KB] = -t.T
    return out


def test_gauss_jordan_schedule_inverts():
    rng = np.random.default_rng(3)
    nc = 90
    np_ = ((nc + KB - 1) // KB) * KB
    Q = rng.standard_normal((nc, nc))
    A = Q @ Q.T + nc * np.eye(nc)
    M = np.eye(np_)
    M[:nc, :nc] = A
    Minv = _gj_schedule(M)
    assert np.allclose(Minv[:nc, :nc], np.linalg.inv(A), rtol=0, atol=1e-10 * np.abs(np.linalg.inv(A)).max())
    assert np.allclose(Minv[nc:, nc:], np.eye(np_ - nc))


def _pcg(A, b, M, rtol, maxit=5000):
    x = np.zeros_like(b)
    r = b.copy()
    z = M(r)
    p = z.copy()
    rz = r @ z
    bb = b @ b
    for it in range(1, maxit + 1):
        q = A @ p
        a = rz / (p @ q)
        x += a * p
        r -= a * q
        if r @ r <= rtol * rtol * bb:
            return it, x
        z = M(r)
        rz2 = r @ z
        p = z + (rz2 / rz) * p
        rz = rz2
    return maxit, x


def test_two_level_cuts_iterations():
    sp, H, pin = _system(nx=24, ny=6, nz=6, ym=1e7)
    n = sp.X.shape[0]
    rowptr, col, blocks = _bsr_pattern(H, n)
    cd = coarse_aggregates(sp.X, ~pin, rowptr, col, box=4)
    P = sps.csr_matrix(_explicit_P(cd["mode"], n, cd["n_agg"]))
    Ac = (P.T @ H @ P).toarray()
    dmax = np.array([Ac[6 * a:6 * a + 6, 6 * a:6 * a + 6].diagonal().max() for a in range(cd["n_agg"])])
    Ac[np.diag_indices_from(Ac)] += np.where(np.repeat(dmax, 6) > 0, 1e-5 * np.repeat(dmax, 6), 1.0)
    Aci = np.linalg.inv(Ac)
    Dinv = np.linalg.inv(blocks[np.concatenate([np.flatnonzero((col == v) & (np.repeat(np.arange(n), np.diff(rowptr)) == v)) for v in range(n)])])
    bj = lambda r: np.einsum("nij,nj->ni", Dinv, r.reshape(-1, 3)).ravel()
    two = lambda r: bj(r) + P @ (Aci @ (P.T @ r))
    rng = np.random.default_rng(0)
    b = rng.standard_normal(3 * n)
    b[pin] = 0.0
    it_bj, x1 = _pcg(H, b, bj, 1e-6)
    it_two, x2 = _pcg(H, b, two, 1e-6)
    assert it_two * 2 < it_bj, (it_bj, it_two)
    assert np.linalg.norm(H @ x2 - b) <= 1e-5 * np.linalg.norm(b)


def _decode_colpack(w):
    w = w.astype(np.int64)
    d = np.stack([((w >> s) & 127) - 64 for s in (0, 7, 14)], 1) / 64.0
    return d, (w >> 21) & 127, (w >> 28) & 7


def test_per_instance_form_two_beams():
    """Per-instance aggregates over a two-mesh batch: local/global aggregate ids, the packed
    column word, dense-block offsets, and each instance's Galerkin block = its own P^T A P."""
    from simkit_gb300.mesh import coarse_aggregates_inst
    parts = [_system(nx=10, ny=4, nz=4, seed=1), _system(nx=6, ny=5, nz=3, ym=3e6, seed=2)]
    Xs = [p[0].X for p in parts]
    Hs = [p[1] for p in parts]
    pins = [p[2] for p in parts]
    rows = np.r_[0, np.cumsum([x.shape[0] for x in Xs])]
    H = sps.block_diag(Hs).tocsr()
    X = np.concatenate(Xs)
    pin = np.concatenate(pins)
    n = X.shape[0]
    rowptr, col, blocks = _bsr_pattern(H, n)
    cd = coarse_aggregates_inst(X, ~pin, rowptr, col, rows, box=4)
    ia = cd["inst_agg"]
    assert ia[0] == 0 and ia[-1] == cd["n_agg"] and np.all(np.diff(ia) <= 127)
    bits = cd["mode"][:, 3].view(np.uint32)
    agg = (bits & 0x1FFFFFFF).astype(np.int64)
    d, local, mask = _decode_colpack(cd["colpack"])
    inst_of = np.repeat(np.arange(len(Xs)), np.diff(rows))
    assert np.array_equal(local, agg - ia[inst_of])
    assert np.array_equal(mask, bits >> 29)
    assert np.array_equal(d.astype(np.float32), cd["mode"][:, :3])        # the same offsets everywhere
    assert np.all(np.abs(cd["mode"][:, :3]) <= 1.0)
    # coarse blocks never couple two instances
    assert np.array_equal(cd["agg_inst"][cd["cb_rc"][0::2]], cd["agg_inst"][cd["cb_rc"][1::2]])
    Ac = _galerkin_blocks(cd, rowptr, col, blocks, n)
    P = _explicit_P(cd["mode"], n, cd["n_agg"])
    ref = P.T @ H.toarray() @ P
    assert np.abs(Ac - ref).max() <= 1e-9 * np.abs(ref).max()
    nps = ((6 * np.diff(ia) + 31) // 32) * 32
    assert np.array_equal(np.diff(cd["inst_moff"]), nps * nps) and cd["max_np"] == nps.max()
