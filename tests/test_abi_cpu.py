"""CPU checks of the native boundary: the library builds, loads and exports
every function the public header declares; the element math the kernels run
(compiled for the host from the same header) agrees with the oracle."""

import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from oracle import psd, snh

HEADER = os.path.join(ROOT, "include", "simkit_gb300.h")
HOST_SRC = os.path.join(ROOT, "tests", "native", "snh_host.cpp")
HOST_SO = os.path.join(ROOT, "tests", "_build", "snh_host.so")


@pytest.fixture(scope="session")
def libpath():
    from simkit_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from simkit_gb300.build import build_library
        build_library()
    return _lib.LIB_PATH


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|int64_t)\s+(skg_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_binding():
    from simkit_gb300 import _lib
    assert set(declared_functions()) == set(_lib.exported_symbols())


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    for name in declared_functions():
        assert hasattr(lib, name), name
    from simkit_gb300 import _lib
    assert _lib.load().skg_version() >= 100


def test_error_path_without_gpu(libpath):
    """Argument validation runs before any device work and reports through skg_last_error."""
    from simkit_gb300 import _lib
    lib = _lib.load()
    assert lib.skg_snh_energy_element_F(4, 0, None, None, None, None, 1, None) == _lib.SKG_ERR_ARG
    assert "dim" in _lib.last_error()
    assert lib.skg_psd_project(None, None, 1, 13, 0, None) == _lib.SKG_ERR_ARG


def test_device_loop_eligibility_without_gpu(libpath):
    """skg_be_plan_eligible is host logic over the mesh and parameter records (no device access):
    the grid PCG forms qualify; profiling, a Newton record, simkit's stop rule, mode 0 and the cluster
    form of meshes up to 24,576 block rows take the host loop; an invalid mesh is not eligible."""
    from simkit_gb300 import _lib
    lib = _lib.load()
    dummy = 256   # non-null placeholders: only sizes, flags and null checks are read

    def mesh(n, coarse=None):
        m = _lib.TetMeshC(n_verts=n, n_tets=6 * n, n_blocks=15 * n, material=0)
        for f in ("tets", "dinv", "dinv32", "vol", "mu", "lam", "mat32", "bsr_rowptr", "bsr_col", "bsr_diag",
                  "bsr_row", "hc_ptr", "hc_src", "v2t_ptr", "v2t"):
            setattr(m, f, dummy)
        if coarse is not None:
            m.coarse = ctypes.pointer(coarse)
        return m

    grid_coarse = _lib.CoarseC(n_agg=475, n_cblocks=1000, mode=dummy, cb_ptr=dummy, cb_slot=dummy, cb_rc=dummy)
    p = _lib.BEParamsC(dt=1.0 / 60.0, tol=1e-6, max_newton=20, precision=_lib.SKG_MIXED, pcg_rtol=-0.25,
                       pcg_max_iter=4000, do_line_search=1, ls_alpha=0.01, ls_beta=0.5, ls_max_iter=100,
                       pcg_mode=3, ls_threshold=-1.0)
    big_two_level, big_one_level, small = mesh(140481, grid_coarse), mesh(140481), mesh(2000)
    assert lib.skg_be_plan_eligible(big_two_level, p) == 1     # mode 3 -> two-level grid form
    assert lib.skg_be_plan_eligible(big_one_level, p) == 1     # mode 3 -> one-level grid form
    assert lib.skg_be_plan_eligible(small, p) == 0             # mode 3 -> one thread-block cluster
    p.pcg_mode = 5
    assert lib.skg_be_plan_eligible(small, p) == 1
    p.pcg_mode = 0
    assert lib.skg_be_plan_eligible(big_one_level, p) == 0     # kernel per phase: host-read stops
    p.pcg_mode = 3
    p.profile = 1
    assert lib.skg_be_plan_eligible(big_two_level, p) == 0
    p.profile = 0
    p.stop_rule = 1
    assert lib.skg_be_plan_eligible(big_two_level, p) == 0
    p.stop_rule = 0
    rec = _lib.NewtonRecordC()
    p.record = ctypes.pointer(rec)
    assert lib.skg_be_plan_eligible(big_two_level, p) == 0
    p.record = None
    assert lib.skg_be_plan_eligible(mesh(0), p) == 0            # sizes the mesh check refuses
    assert lib.skg_be_plan_create(big_two_level, p, None, None, None) == _lib.SKG_ERR_ARG


def test_pattern_builder_matches_scipy():
    """The host pattern builder reproduces scipy's pattern of J^T blockdiag(He) J."""
    from simkit_gb300 import _lib
    from simkit_gb300.beams import make_beam
    from oracle import fem
    lib = _lib.load()
    b = make_beam(3, 2, 4, jitter=0.1, seed=2)
    T = np.ascontiguousarray(b.T.astype(np.int32))
    n, t = b.n_verts, b.n_tets
    nb = ctypes.c_int64()
    a = lambda x: x.ctypes.data_as(ctypes.c_void_p)
    assert lib.skg_pattern_build(a(T), n, t, ctypes.byref(nb), None, None, None, None, None, None, None) == 0
    nb = nb.value
    rp = np.empty(n + 1, np.int32); col = np.empty(nb, np.int32); dg = np.empty(n, np.int32)
    hp = np.empty(nb + 1, np.int32); hs = np.empty(16 * t, np.int32)
    vp = np.empty(n + 1, np.int32); vt = np.empty(4 * t, np.int32)
    assert lib.skg_pattern_build(a(T), n, t, ctypes.byref(ctypes.c_int64()), a(rp), a(col), a(dg), a(hp), a(hs),
                                 a(vp), a(vt)) == 0
    J = fem.deformation_jacobian(b.X, b.T)
    x = b.X + 1e-3 * np.random.default_rng(0).standard_normal(b.X.shape)
    K = snh.hessian_x(x, J, b.mu, b.lam, fem.tet_volumes(b.X, b.T))
    K.sort_indices()
    # expand blocks to scalars
    rows = []
    for v in range(n):
        for i in range(3):
            rows.append(np.concatenate([[3 * c, 3 * c + 1, 3 * c + 2] for c in col[rp[v]:rp[v + 1]]]))
    indptr = np.concatenate([[0], np.cumsum([r.size for r in rows])])
    assert np.array_equal(indptr, K.indptr)
    assert np.array_equal(np.concatenate(rows), K.indices)
    assert np.all(col[dg] == np.arange(n))
    # every (tet, a, b) block appears exactly once, lists ordered by tet
    assert hp[-1] == 16 * t and np.all(np.diff(hp) > 0)
    for s in range(nb):
        tets = hs[hp[s]:hp[s + 1]] >> 4
        assert np.all(np.diff(tets) > 0)
    assert vp[-1] == 4 * t


def test_pattern_rejects_bad_tets():
    from simkit_gb300 import _lib
    lib = _lib.load()
    T = np.array([[0, 1, 1, 2]], np.int32)
    nb = ctypes.c_int64()
    assert lib.skg_pattern_build(T.ctypes.data_as(ctypes.c_void_p), 3, 1, ctypes.byref(nb), None, None, None,
                                 None, None, None, None) == _lib.SKG_ERR_ARG
    T = np.array([[0, 1, 2, 7]], np.int32)
    assert lib.skg_pattern_build(T.ctypes.data_as(ctypes.c_void_p), 4, 1, ctypes.byref(nb), None, None, None,
                                 None, None, None, None) == _lib.SKG_ERR_ARG


# ------------------------------------------------- host build of the kernels' math
@pytest.fixture(scope="session")
def hostmath():
    os.makedirs(os.path.dirname(HOST_SO), exist_ok=True)
    if not os.path.exists(HOST_SO) or os.path.getmtime(HOST_SO) < max(
            os.path.getmtime(HOST_SRC), os.path.getmtime(os.path.join(ROOT, "simkit_gb300", "csrc", "snh_math.cuh"))):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", HOST_SO, HOST_SRC])
    return ctypes.CDLL(HOST_SO)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _cases(rng, t=300):
    F = np.eye(3)[None] + np.concatenate([0.05 * rng.standard_normal((t // 4, 3, 3)),
                                          0.3 * rng.standard_normal((t // 4, 3, 3)),
                                          1.0 * rng.standard_normal((t // 4, 3, 3)),
                                          0.2 * rng.standard_normal((t - 3 * (t // 4), 3, 3))])
    F[3 * (t // 4):, :, 0] *= -1.0       # inverted elements
    ym = np.exp(rng.uniform(np.log(1e5), np.log(1e7), t))
    pr = rng.uniform(0.3, 0.49, t)
    mu, lam = ym / (2 * (1 + pr)), ym * pr / ((1 + pr) * (1 - 2 * pr))
    vol = rng.uniform(1e-7, 5e-6, t)
    X = rng.standard_normal((t, 4, 3))
    E = (X[:, 1:] - X[:, [0]]).transpose(0, 2, 1)
    Dinv = np.linalg.inv(E)
    gN = np.empty((t, 4, 3))
    gN[:, 1:] = Dinv
    gN[:, 0] = -Dinv.sum(1)
    return np.ascontiguousarray(F), mu, lam, vol, np.ascontiguousarray(gN)


def _unpack78(o):
    t = o.shape[0]
    K = np.zeros((t, 12, 12))
    iu = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    for a in range(4):
        for n_, (i, k) in enumerate(iu):
            K[:, 3 * a + i, 3 * a + k] = o[:, 6 * a + n_]
            K[:, 3 * a + k, 3 * a + i] = o[:, 6 * a + n_]
    for q, (a, b) in enumerate([(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]):
        blk = o[:, 24 + 9 * q:33 + 9 * q].reshape(t, 3, 3)
        K[:, 3 * a:3 * a + 3, 3 * b:3 * b + 3] = blk
        K[:, 3 * b:3 * b + 3, 3 * a:3 * a + 3] = blk.transpose(0, 2, 1)
    return K


def lifted_oracle(F, mu, lam, vol, gN):
    H9p = psd.psd_project(snh.hessian_element_F(F, mu, lam) * vol[:, None, None])
    t = F.shape[0]
    return np.einsum("taj,tbl,tijkl->taibk", gN, gN, H9p.reshape(t, 3, 3, 3, 3)).reshape(t, 12, 12)


@pytest.mark.parametrize("prec,tol", [(64, 1e-12), (32, 3e-6)])
def test_tet_hessian_analytic_psd_matches_eigh_floor(hostmath, prec, tol):
    """Analytic-eigensystem PSD floor + 12x12 lift == simkit's eigh floor of vol*He, lifted."""
    rng = np.random.default_rng(5)
    F, mu, lam, vol, gN = _cases(rng)
    t = F.shape[0]
    out = np.zeros((t, 78))
    hostmath.h_tet_hessian(prec, ctypes.c_int64(t), _p(F), _p(mu), _p(lam), _p(vol), _p(gN), _p(out),
                           ctypes.c_double(0.1))
    K = _unpack78(out)
    Ko = lifted_oracle(F, mu, lam, vol, gN)
    err = np.abs(K - Ko).max(axis=(1, 2)) / np.abs(Ko).max(axis=(1, 2))
    assert err.max() < tol


@pytest.mark.parametrize("prec,tol", [(64, 1e-12), (32, 3e-6)])
def test_mmnh_tet_hessian_analytic_psd_matches_eigh_floor(hostmath, prec, tol):
    """The same analytic PSD floor + lift with the Macklin-Mueller coefficients (A = mu, B = 0,
    D = lam (J - 1) - mu) == eigh floor of the oracle's vol * He, lifted."""
    from oracle import mmnh
    rng = np.random.default_rng(15)
    F, mu, lam, vol, gN = _cases(rng)
    t = F.shape[0]
    out = np.zeros((t, 78))
    hostmath.h_tet_hessian_mat(prec, 1, ctypes.c_int64(t), _p(F), _p(mu), _p(lam), _p(vol), _p(gN), _p(out),
                               ctypes.c_double(0.1))
    K = _unpack78(out)
    H9p = psd.psd_project(mmnh.hessian_element_F(F, mu, lam) * vol[:, None, None])
    Ko = np.einsum("taj,tbl,tijkl->taibk", gN, gN, H9p.reshape(t, 3, 3, 3, 3)).reshape(t, 12, 12)
    err = np.abs(K - Ko).max(axis=(1, 2)) / np.abs(Ko).max(axis=(1, 2))
    assert err.max() < tol


def test_mmnh_element_math_matches_oracle(hostmath):
    """Direct and displacement forms of the Macklin-Mueller energy and stress, and its F-Hessian."""
    from oracle import mmnh
    rng = np.random.default_rng(16)
    t = 200
    G = np.concatenate([1e-4 * rng.standard_normal((t // 2, 3, 3)), 0.2 * rng.standard_normal((t // 2, 3, 3))])
    F = np.ascontiguousarray(np.eye(3)[None] + G)
    G = np.ascontiguousarray(G)
    mu = rng.uniform(3e4, 3e6, t)
    lam = mu * rng.uniform(1.5, 40, t)
    psi, dpsi, P, Pd, H = np.zeros(t), np.zeros(t), np.zeros((t, 9)), np.zeros((t, 9)), np.zeros((t, 81))
    hostmath.h_mm(64, ctypes.c_int64(t), _p(F), _p(G), _p(mu), _p(lam), _p(psi), _p(dpsi), _p(P), _p(Pd), _p(H))
    po = mmnh.energy_element_F(F, mu, lam).ravel()
    Po = mmnh.gradient_element_F(F, mu, lam).reshape(t, 9)
    Ho = mmnh.hessian_element_F(F, mu, lam).reshape(t, 81)
    scale = mu + lam
    assert np.all(np.abs(psi - po) <= 1e-12 * scale)
    assert np.all(np.abs(dpsi - po) <= 1e-9 * np.abs(po) + 1e-15 * scale)     # psi(I) = 0
    assert np.all(np.abs(P - Po).max(1) <= 1e-12 * scale)
    assert np.all(np.abs(Pd - Po).max(1) <= 1e-9 * np.abs(Po).max(1) + 1e-15 * scale)
    assert np.all(np.abs(H - Ho).max(1) <= 1e-12 * scale)
    # FP32 displacement forms keep relative accuracy near rest
    d32, P32 = np.zeros(t), np.zeros((t, 9))
    psi32, H32, Pf = np.zeros(t), np.zeros((t, 81)), np.zeros((t, 9))
    hostmath.h_mm(32, ctypes.c_int64(t), _p(F), _p(G), _p(mu), _p(lam), _p(psi32), _p(d32), _p(Pf), _p(P32), _p(H32))
    assert np.max(np.abs(d32 - dpsi) / np.abs(dpsi)) < 2e-5
    assert np.max(np.abs(P32 - Pd).max(1) / np.abs(Pd).max(1)) < 2e-5


@pytest.mark.parametrize("mat,name", [(2, "arap"), (3, "fcr")])
@pytest.mark.parametrize("prec,tol", [(64, 1e-12), (32, 3e-6)])
def test_corot_tet_hessian_analytic_psd_matches_eigh_floor(hostmath, mat, name, prec, tol):
    """ARAP / fixed-corotated per-tet Hessian: the analytic terms plus the three rank-1 twist
    terms of dR/dF, with the eigenvalue floor on the twist eigenvalues, == eigh floor of the
    oracle's vol * He (including inverted elements), lifted to 12 x 12."""
    from oracle import corot
    rng = np.random.default_rng(25 + mat)
    F, mu, lam, vol, gN = _cases(rng)
    t = F.shape[0]
    out = np.zeros((t, 78))
    hostmath.h_tet_hessian_mat(prec, mat, ctypes.c_int64(t), _p(F), _p(mu), _p(lam), _p(vol), _p(gN), _p(out),
                               ctypes.c_double(0.1))
    K = _unpack78(out)
    He = corot.arap_hessian_element_F(F, mu) if name == "arap" else corot.fcr_hessian_element_F(F, mu, lam)
    H9p = psd.psd_project(He * vol[:, None, None])
    Ko = np.einsum("taj,tbl,tijkl->taibk", gN, gN, H9p.reshape(t, 3, 3, 3, 3)).reshape(t, 12, 12)
    err = np.abs(K - Ko).max(axis=(1, 2)) / np.abs(Ko).max(axis=(1, 2))
    assert err.max() < tol


@pytest.mark.parametrize("mat,name", [(2, "arap"), (3, "fcr")])
def test_corot_element_math_matches_oracle(hostmath, mat, name):
    """Direct and displacement forms of the ARAP / fixed-corotated energy and stress, the
    F-Hessian, and the 2D element tier; the FP32 displacement-form energy keeps relative
    accuracy from rest (|G| = 1e-5) to inverted elements."""
    from oracle import corot
    rng = np.random.default_rng(30 + mat)
    t = 400
    G = np.concatenate([1e-5 * rng.standard_normal((t // 4, 3, 3)), 1e-3 * rng.standard_normal((t // 4, 3, 3)),
                        0.2 * rng.standard_normal((t // 4, 3, 3)), 0.3 * rng.standard_normal((t // 4, 3, 3))])
    G[3 * t // 4:, :, 0] -= 2.0 * (np.eye(3)[None] + G[3 * t // 4:])[:, :, 0]   # inverted: F[:, :, 0] negated
    G = np.ascontiguousarray(G)
    F = np.ascontiguousarray(np.eye(3)[None] + G)
    assert (np.linalg.det(F[3 * t // 4:]) < 0).mean() > 0.9
    mu = rng.uniform(3e4, 3e6, t)
    lam = mu * rng.uniform(1.5, 40, t)
    res = {}
    for prec in (64, 32):
        r = np.zeros(t), np.zeros(t), np.zeros((t, 9)), np.zeros((t, 9)), np.zeros((t, 81))
        hostmath.h_mat(prec, mat, ctypes.c_int64(t), _p(F), _p(G), _p(mu), _p(lam), *map(_p, r))
        res[prec] = r
    psi, dpsi, P, Pd, H = res[64]
    if name == "arap":
        po, Po, Ho = (corot.arap_energy_element_F(F, mu).ravel(), corot.arap_gradient_element_F(F, mu).reshape(t, 9),
                      corot.arap_hessian_element_F(F, mu).reshape(t, 81))
    else:
        po, Po, Ho = (corot.fcr_energy_element_F(F, mu, lam).ravel(),
                      corot.fcr_gradient_element_F(F, mu, lam).reshape(t, 9),
                      corot.fcr_hessian_element_F(F, mu, lam).reshape(t, 81))
    scale = mu + lam
    assert np.all(np.abs(psi - po) <= 1e-12 * scale)
    # the oracle's |F - R|^2 from absolute F carries ~1e-16 absolute error: near rest the
    # displacement form is the more accurate of the two
    assert np.all(np.abs(dpsi - po) <= 1e-9 * np.abs(po) + 1e-14 * scale)
    assert np.all(np.abs(P - Po).max(1) <= 1e-12 * scale)
    assert np.all(np.abs(Pd - Po).max(1) <= 1e-9 * np.abs(Po).max(1) + 1e-14 * scale)
    assert np.all(np.abs(H - Ho).max(1) <= 1e-11 * scale)
    d32 = res[32][1]
    assert np.max(np.abs(d32 - dpsi) / np.abs(dpsi)) < 1e-5
    # 2D element tier
    F2 = np.ascontiguousarray(np.eye(2)[None] + 0.4 * rng.standard_normal((t, 2, 2)))
    psi2, P2, H2 = np.zeros(t), np.zeros((t, 4)), np.zeros((t, 16))
    hostmath.h_mat2(64, mat, ctypes.c_int64(t), _p(F2), _p(mu), _p(lam), _p(psi2), _p(P2), _p(H2))
    if name == "arap":
        po, Po, Ho = corot.arap_energy_element_F(F2, mu), corot.arap_gradient_element_F(F2, mu), \
            corot.arap_hessian_element_F(F2, mu)
    else:
        po, Po, Ho = corot.fcr_energy_element_F(F2, mu, lam), corot.fcr_gradient_element_F(F2, mu, lam), \
            corot.fcr_hessian_element_F(F2, mu, lam)
    assert np.all(np.abs(psi2 - po.ravel()) <= 1e-12 * scale)
    assert np.all(np.abs(P2 - Po.reshape(t, 4)).max(1) <= 1e-12 * scale)
    assert np.all(np.abs(H2 - Ho.reshape(t, 16)).max(1) <= 1e-11 * scale)


@pytest.mark.parametrize("mat", [0, 1])
def test_double_float_stress_matches_fp64(hostmath, mat):
    """The double-float displacement-form stress (dfloat.cuh) of the mixed-precision force kernel
    agrees with the FP64 evaluation to ~1e-13 of the element's stress, from |G| = 1e-6 to 0.4."""
    rng = np.random.default_rng(40 + mat)
    t = 800
    G = np.concatenate([s * rng.standard_normal((t // 4, 9)) for s in (1e-6, 1e-3, 0.1, 0.4)])
    G = np.ascontiguousarray(G)
    F = np.ascontiguousarray(G + np.eye(3).reshape(1, 9))
    mu = rng.uniform(3e4, 3e6, t)
    lam = mu * rng.uniform(1.5, 40, t)
    r = np.zeros(t), np.zeros(t), np.zeros((t, 9)), np.zeros((t, 9)), np.zeros((t, 81))
    hostmath.h_mat(64, mat, ctypes.c_int64(t), _p(F), _p(G), _p(mu), _p(lam), *map(_p, r))
    Pd = r[3]
    Pf = np.zeros((t, 9))
    hostmath.h_pk1_disp_df(mat, ctypes.c_int64(t), _p(G), _p(mu), _p(lam), _p(Pf))
    rel = np.abs(Pf - Pd).max(1) / np.abs(Pd).max(1)
    assert rel[: 3 * t // 4].max() < 1e-13
    assert rel.max() < 3e-12


def test_le_element_math_and_tet_stiffness_match_oracle(hostmath):
    """Linear elasticity: element math (direct, displacement and 2D forms) and the per-tet
    stiffness J^T (vol H) J, never projected (linear_elasticity.py:43-230)."""
    from oracle import linel
    rng = np.random.default_rng(50)
    F, mu, lam, vol, gN = _cases(rng)
    t = F.shape[0]
    G = np.ascontiguousarray(F - np.eye(3)[None])
    r = np.zeros(t), np.zeros(t), np.zeros((t, 9)), np.zeros((t, 9)), np.zeros((t, 81))
    hostmath.h_mat(64, 4, ctypes.c_int64(t), _p(F), _p(G), _p(mu), _p(lam), *map(_p, r))
    po = linel.energy_element_F(F, mu, lam).ravel()
    Po = linel.gradient_element_F(F, mu, lam).reshape(t, 9)
    Ho = linel.hessian_element_F(F, mu, lam)
    scale = mu + lam
    assert np.all(np.abs(r[0] - po) <= 1e-13 * scale) and np.all(np.abs(r[1] - po) <= 1e-13 * scale)
    assert np.all(np.abs(r[2] - Po).max(1) <= 1e-13 * scale) and np.all(np.abs(r[3] - Po).max(1) <= 1e-13 * scale)
    assert np.array_equal(r[4], Ho.reshape(t, 81))
    F2 = np.ascontiguousarray(F[:, :2, :2])
    p2, P2, H2 = np.zeros(t), np.zeros((t, 4)), np.zeros((t, 16))
    hostmath.h_mat2(64, 4, ctypes.c_int64(t), _p(F2), _p(mu), _p(lam), _p(p2), _p(P2), _p(H2))
    assert np.all(np.abs(p2 - linel.energy_element_F(F2, mu, lam).ravel()) <= 1e-13 * scale)
    assert np.all(np.abs(P2 - linel.gradient_element_F(F2, mu, lam).reshape(t, 4)).max(1) <= 1e-13 * scale)
    for prec, tol in ((64, 1e-14), (32, 1e-6)):
        out = np.zeros((t, 78))
        hostmath.h_tet_hessian_mat(prec, 4, ctypes.c_int64(t), _p(F), _p(mu), _p(lam), _p(vol), _p(gN), _p(out),
                                   ctypes.c_double(0.1))
        K = _unpack78(out)
        Ko = np.einsum("taj,tbl,tijkl->taibk", gN, gN,
                       (Ho * vol[:, None, None]).reshape(t, 3, 3, 3, 3)).reshape(t, 12, 12)
        err = np.abs(K - Ko).max(axis=(1, 2)) / np.abs(Ko).max(axis=(1, 2))
        assert err.max() < tol


def test_displacement_forms_match_oracle(hostmath):
    rng = np.random.default_rng(6)
    t = 200
    G = np.concatenate([1e-4 * rng.standard_normal((t // 2, 3, 3)), 0.1 * rng.standard_normal((t // 2, 3, 3))])
    mu = rng.uniform(3e4, 3e6, t)
    lam = mu * rng.uniform(1.5, 40, t)
    d64, P64 = np.zeros(t), np.zeros((t, 9))
    hostmath.h_disp(64, ctypes.c_int64(t), _p(np.ascontiguousarray(G)), _p(mu), _p(lam), _p(d64), _p(P64))
    F = np.eye(3)[None] + G
    rest = snh.energy_element_F(np.repeat(np.eye(3)[None], t, 0), mu, lam).ravel()
    dpsi = snh.energy_element_F(F, mu, lam).ravel() - rest
    # the oracle's difference of two O(mu) numbers is itself only good to ~1e-16 |rest|
    assert np.all(np.abs(d64 - dpsi) <= 1e-9 * np.abs(dpsi) + 1e-15 * np.abs(rest))
    Po = snh.gradient_element_F(F, mu, lam).reshape(t, 9)
    assert np.all(np.abs(P64 - Po).max(1) <= 1e-9 * np.abs(Po).max(1) + 1e-15 * mu)
    # FP32: relative to the element's own scale
    d32, P32 = np.zeros(t), np.zeros((t, 9))
    hostmath.h_disp(32, ctypes.c_int64(t), _p(np.ascontiguousarray(G)), _p(mu), _p(lam), _p(d32), _p(P32))
    assert np.max(np.abs(d32 - d64) / np.abs(d64)) < 2e-5
    assert np.max(np.abs(P32 - P64).max(1) / np.abs(P64).max(1)) < 2e-5


def test_svd_rotation_variant(hostmath):
    rng = np.random.default_rng(7)
    F, *_ = _cases(rng, 200)
    t = F.shape[0]
    for prec, tol in ((64, 1e-12), (32, 2e-5)):
        U, s, V = np.zeros((t, 9)), np.zeros((t, 3)), np.zeros((t, 9))
        hostmath.h_svd(prec, ctypes.c_int64(t), _p(F), _p(U), _p(s), _p(V))
        U, V = U.reshape(t, 3, 3), V.reshape(t, 3, 3)
        R = U @ (s[:, :, None] * V.transpose(0, 2, 1))
        assert np.abs(R - F).max() < tol * np.abs(F).max() * 10
        assert np.allclose(np.linalg.det(U), 1, atol=1e-4) and np.allclose(np.linalg.det(V), 1, atol=1e-4)
        assert np.all(s[:, 0] >= s[:, 1] - 1e-6) and np.all(s[:, 1] >= np.abs(s[:, 2]) - 1e-6)
        assert np.all(np.sign(s[:, 2]) == np.sign(np.linalg.det(F)))
