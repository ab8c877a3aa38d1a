"""simkit-compatible entry points of the FEM path, computed on the GPU.

Each function keeps the signature, argument meaning, return types and error
behaviour of the simkit function it replaces (cited per function).  numpy
inputs give numpy / scipy outputs, like simkit; torch CUDA tensors stay on the
device.  All arithmetic runs in the CUDA library (``_lib``); there is no CPU
fallback - without the library every call raises.
"""

from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np
import scipy.sparse as sps
import torch

from . import _lib
from ._lib import SKG_FP64, SKG_MIXED, check
from .mesh import TetMesh, _ptr, _stream_ptr

_PREC = {"fp64": SKG_FP64, "mixed": SKG_MIXED, "fp32": SKG_MIXED}


def _dev(a):
    """FP64 contiguous CUDA tensor from a numpy array, list or tensor."""
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda", dtype=torch.float64).contiguous()
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64))).to("cuda")


def _out(t: torch.Tensor, like):
    return t if isinstance(like, torch.Tensor) else t.cpu().numpy()


# --------------------------------------------------------------------------- #
# element tier: simkit/energies/stable_neo_hookean.py:65-443                  #
# --------------------------------------------------------------------------- #
def _elem(fn, F, mu, lam, shape_of, precision, name="Stable Neo-Hookean"):
    d = F.shape[-1]
    if d not in (2, 3):
        raise ValueError(f"{name} supports dim=2 or dim=3")
    Fd = _dev(F).reshape(-1, d, d)
    t = Fd.shape[0]
    mud = _dev(mu).reshape(-1)
    lamd = _dev(lam).reshape(-1)
    out = torch.empty(shape_of(t, d), dtype=torch.float64, device="cuda")
    check(getattr(_lib.load(), fn)(d, _PREC[precision], _ptr(Fd), _ptr(mud), _ptr(lamd), _ptr(out), t, _stream_ptr()))
    return _out(out, F)


def stable_neo_hookean_energy_element_F(F, mu, lam, precision: str = "fp64"):
    """psi per element, (t, 1).  simkit ``stable_neo_hookean_energy_element_F`` (snh.py:65-129)."""
    return _elem("skg_snh_energy_element_F", F, mu, lam, lambda t, d: (t, 1), precision)


def stable_neo_hookean_gradient_element_F(F, mu, lam, precision: str = "fp64"):
    """PK1 per element, (t, d, d).  simkit ``stable_neo_hookean_gradient_element_F`` (snh.py:132-218)."""
    return _elem("skg_snh_gradient_element_F", F, mu, lam, lambda t, d: (t, d, d), precision)


def stable_neo_hookean_hessian_element_F(F, mu, lam, precision: str = "fp64"):
    """(t, d*d, d*d) unprojected blocks.  simkit ``stable_neo_hookean_hessian_element_F`` (snh.py:221-443)."""
    return _elem("skg_snh_hessian_element_F", F, mu, lam, lambda t, d: (t, d * d, d * d), precision)


# --------------------------------------------------------------------------- #
# psd_project: simkit/psd_project.py:12-47                                    #
# --------------------------------------------------------------------------- #
def psd_project(H, method: str = "proj"):
    """Floor (``'proj'``, 1e-6) or take |.| (``'abs'``) of each block's eigenvalues."""
    if method not in ("proj", "abs"):
        raise ValueError("method must be 'proj' or 'abs'")
    Hd = _dev(H)
    if Hd.ndim == 2:
        Hd = Hd[None]
    n, d, _ = Hd.shape
    out = torch.empty_like(Hd)
    check(_lib.load().skg_psd_project(_ptr(Hd), _ptr(out), n, d, 0 if method == "proj" else 1, _stream_ptr()))
    return _out(out, H)


# --------------------------------------------------------------------------- #
# deformation Jacobian as a device operator                                   #
# --------------------------------------------------------------------------- #
class DeformationJacobian:
    """The per-tet operator behind simkit's sparse J (deformation_jacobian.py:9-87).

    ``J @ x`` gives the stacked F (9t, 1); ``J.T @ y`` gives the vertex gather
    (3n, 1); ``to_scipy()`` builds the same csc matrix simkit returns.
    """

    def __init__(self, X, T):
        X = np.asarray(X, dtype=np.float64)
        T = np.asarray(T)
        if X.shape[1] != 3 or T.shape[1] != 4:
            raise ValueError("the GPU deformation Jacobian supports tetrahedra in 3D")
        self.mesh = TetMesh(X, T, np.ones(T.shape[0]), np.ones(T.shape[0]))
        self.shape = (9 * T.shape[0], 3 * X.shape[0])

    @property
    def T(self):
        return _Transposed(self)

    def transpose(self):
        return _Transposed(self)

    def __matmul__(self, x):
        m = self.mesh
        xd = _dev(x).reshape(-1)
        if xd.numel() != 3 * m.n:
            raise ValueError("dimension mismatch")
        F = torch.empty(9 * m.t, dtype=torch.float64, device="cuda")
        check(_lib.load().skg_tet_deformation_gradient(_ptr(m.tets), _ptr(m.dinv), _ptr(xd), m.t, _ptr(F),
                                                       _stream_ptr()))
        return _out(F.reshape(-1, 1), x)

    def to_scipy(self) -> sps.csc_matrix:
        m = self.mesh
        t = m.t
        D = m.dinv.cpu().numpy().reshape(9, t).T.reshape(t, 3, 3)    # rows = grad N_1..3
        G = np.empty((t, 4, 3))
        G[:, 1:] = D
        G[:, 0] = -D.sum(axis=1)
        T = m.T_host.astype(np.int64)
        e = np.arange(t)[:, None, None, None]
        i = np.arange(3)[None, :, None, None]
        j = np.arange(3)[None, None, :, None]
        rows = np.broadcast_to(9 * e + 3 * i + j, (t, 3, 3, 4))
        cols = np.broadcast_to(3 * T[:, None, None, :] + i, (t, 3, 3, 4))
        vals = np.broadcast_to(G.transpose(0, 2, 1)[:, None, :, :], (t, 3, 3, 4))
        J = sps.csc_matrix((vals.ravel(), (rows.ravel(), cols.ravel())), shape=self.shape)
        J.eliminate_zeros()
        return J

    tocsc = to_scipy


class _Transposed:
    def __init__(self, J):
        self.J = J
        self.shape = (J.shape[1], J.shape[0])

    def __matmul__(self, y):
        m = self.J.mesh
        yd = _dev(y).reshape(-1)
        if yd.numel() != 9 * m.t:
            raise ValueError("dimension mismatch")
        out = torch.empty(3 * m.n, dtype=torch.float64, device="cuda")
        check(_lib.load().skg_tet_gradient_scatter(_ptr(m.tets), _ptr(m.dinv), _ptr(yd), _ptr(m.v2t_ptr),
                                                   _ptr(m.v2t), m.n, m.t, _ptr(out), _stream_ptr()))
        return _out(out.reshape(-1, 1), y)


def deformation_jacobian(X, T) -> DeformationJacobian:
    """GPU operator for simkit ``deformation_jacobian`` (deformation_jacobian.py:9-87)."""
    return DeformationJacobian(X, T)


def volume(X, T):
    """Signed tet volumes (t, 1).  simkit ``volume`` (volume.py:14-41) for tets."""
    T = np.asarray(T)
    if T.shape[1] != 4:
        raise ValueError("the GPU volume supports tetrahedra")
    Xd = _dev(X).reshape(-1)
    Td = torch.from_numpy(np.ascontiguousarray(T.astype(np.int32))).cuda()
    t = T.shape[0]
    dinv = torch.empty(9 * t, dtype=torch.float64, device="cuda")
    vol = torch.empty(t, dtype=torch.float64, device="cuda")
    check(_lib.load().skg_tet_setup(_ptr(Xd), _ptr(Td), Xd.numel() // 3, t, _ptr(dinv), _ptr(vol), _stream_ptr()))
    return _out(vol.reshape(-1, 1), X)


# --------------------------------------------------------------------------- #
# assembled tier: simkit/energies/stable_neo_hookean.py:449-538               #
# --------------------------------------------------------------------------- #
def _operator(J) -> TetMesh:
    if isinstance(J, DeformationJacobian):
        return J.mesh
    raise TypeError("pass the operator returned by simkit_gb300.deformation_jacobian")


def _bind(J, mu, lam, vol, material=0) -> TetMesh:
    m = _operator(J)
    m.set_material(mu, lam, vol)
    m.set_energy(material)
    return m


def stable_neo_hookean_energy_x(X, J, mu, lam, vol) -> float:
    """sum vol psi(J x).  simkit ``stable_neo_hookean_energy_x`` (snh.py:449-474)."""
    m = _bind(J, mu, lam, vol)
    x = _dev(X).reshape(-1)
    ws = m.workspace(SKG_FP64)
    e = ctypes.c_double()
    check(_lib.load().skg_snh_energy_x(ctypes.byref(m.c), _ptr(x), ctypes.byref(e), _ptr(ws), _stream_ptr()))
    return float(e.value)


def stable_neo_hookean_gradient_x(X, J, mu, lam, vol):
    """J^T vec(vol P), (3n, 1).  simkit ``stable_neo_hookean_gradient_x`` (snh.py:477-503)."""
    m = _bind(J, mu, lam, vol)
    x = _dev(X).reshape(-1)
    ws = m.workspace(SKG_FP64)
    g = torch.empty(3 * m.n, dtype=torch.float64, device="cuda")
    check(_lib.load().skg_snh_gradient_x(ctypes.byref(m.c), _ptr(x), _ptr(g), _ptr(ws), _stream_ptr()))
    return _out(g.reshape(-1, 1), X)


def assemble_hessian_blocks(mesh: TetMesh, X, precision="fp64", psd=True) -> torch.Tensor:
    """Block values (entry-major layout) of J^T blockdiag(psd(vol He)) J on the device."""
    prec = _PREC[precision]
    x = _dev(X).reshape(-1)
    ws = mesh.workspace(prec)
    if prec == SKG_FP64:
        val = torch.empty(9 * mesh.nb, dtype=torch.float64, device="cuda")
        check(_lib.load().skg_snh_hessian_x(ctypes.byref(mesh.c), _ptr(x), prec, int(psd), _ptr(val), None, _ptr(ws),
                                            _stream_ptr()))
    else:
        val = torch.empty(9 * mesh.nb, dtype=torch.float32, device="cuda")
        check(_lib.load().skg_snh_hessian_x(ctypes.byref(mesh.c), _ptr(x), prec, int(psd), None, _ptr(val), _ptr(ws),
                                            _stream_ptr()))
    return val


class BlockMatrix:
    """Assembled 3x3-block symmetric matrix resident on the GPU.  ``+`` a diagonal matrix (scipy or
    dense, e.g. a lumped M / h^2) or a BlockMatrix of the same mesh, ``*`` or ``/`` a scalar stay on the
    device; ``+`` any other matrix gives the host sum."""

    def __init__(self, mesh: TetMesh, val: torch.Tensor):
        self.mesh = mesh
        self.val = val
        self.shape = (3 * mesh.n, 3 * mesh.n)

    def to_scipy(self) -> sps.csr_matrix:
        return self.mesh.block_values_to_csr(self.val)

    def __add__(self, other):
        if isinstance(other, BlockMatrix):
            if other.mesh is not self.mesh:
                raise ValueError("BlockMatrix sum needs both matrices on the same mesh")
            return BlockMatrix(self.mesh, self.val + other.val.to(self.val.dtype))
        d = _diagonal_of(other, self.shape[0])
        if d is None:
            return self.to_scipy() + other
        val = self.val.clone()
        val[self.mesh.diag_value_index()] += torch.from_numpy(d).to(device=val.device, dtype=val.dtype)
        return BlockMatrix(self.mesh, val)

    __radd__ = __add__

    def __mul__(self, s):
        if not np.isscalar(s):
            return NotImplemented
        return BlockMatrix(self.mesh, self.val * float(s))

    __rmul__ = __mul__

    def __truediv__(self, s):
        if not np.isscalar(s):
            return NotImplemented
        return BlockMatrix(self.mesh, self.val / float(s))

    tocsr = to_scipy

    def tocsc(self):
        return self.to_scipy().tocsc()


def stable_neo_hookean_hessian_x(X, J, mu, lam, vol, psd: bool = True, precision: str = "fp64"):
    """J^T blockdiag(psd(vol He)) J.  simkit ``stable_neo_hookean_hessian_x`` (snh.py:506-538).

    numpy input returns a scipy sparse matrix like simkit; torch input returns
    a device ``BlockMatrix``.
    """
    m = _bind(J, mu, lam, vol)
    val = assemble_hessian_blocks(m, X, precision=precision, psd=psd)
    B = BlockMatrix(m, val)
    return B if isinstance(X, torch.Tensor) else B.to_scipy()


def stable_neo_hookean_energy(X, T, mu, lam, U: Optional[np.ndarray] = None) -> float:
    """simkit ``stable_neo_hookean_energy`` (snh.py:654-679)."""
    J = deformation_jacobian(X, T)
    return stable_neo_hookean_energy_x(X if U is None else U, J, mu, lam, volume(X, T))


def stable_neo_hookean_gradient(X, T, mu, lam, U: Optional[np.ndarray] = None):
    """simkit ``stable_neo_hookean_gradient`` (snh.py:682-707)."""
    J = deformation_jacobian(X, T)
    return stable_neo_hookean_gradient_x(X if U is None else U, J, mu, lam, volume(X, T))


def stable_neo_hookean_hessian(X, T, mu, lam, U: Optional[np.ndarray] = None, psd: bool = True):
    """simkit ``stable_neo_hookean_hessian`` (snh.py:710-737)."""
    J = deformation_jacobian(X, T)
    return stable_neo_hookean_hessian_x(X if U is None else U, J, mu, lam, volume(X, T), psd=psd)


# --------------------------------------------------------------------------- #
# Macklin-Mueller neo-Hookean: simkit/energies/macklin_mueller_neo_hookean.py  #
# --------------------------------------------------------------------------- #
_MM = "Macklin-Mueller Neo-Hookean"
MATERIALS = {"stable-neo-hookean": 0, "macklin-mueller-neo-hookean": 1, "arap": 2, "fcr": 3, "linear-elasticity": 4}


def macklin_mueller_neo_hookean_energy_element_F(F, mu, lam, precision: str = "fp64"):
    """psi per element, (t, 1).  simkit ``macklin_mueller_neo_hookean_energy_element_F`` (:66-122)."""
    return _elem("skg_mmnh_energy_element_F", F, mu, lam, lambda t, d: (t, 1), precision, _MM)


def macklin_mueller_neo_hookean_gradient_element_F(F, mu, lam, precision: str = "fp64"):
    """PK1 per element, (t, d, d).  simkit ``macklin_mueller_neo_hookean_gradient_element_F`` (:125-185)."""
    return _elem("skg_mmnh_gradient_element_F", F, mu, lam, lambda t, d: (t, d, d), precision, _MM)


def macklin_mueller_neo_hookean_hessian_element_F(F, mu, lam, precision: str = "fp64"):
    """(t, d*d, d*d) unprojected blocks.  simkit ``macklin_mueller_neo_hookean_hessian_element_F`` (:188-374)."""
    return _elem("skg_mmnh_hessian_element_F", F, mu, lam, lambda t, d: (t, d * d, d * d), precision, _MM)


def macklin_mueller_neo_hookean_energy_x(X, J, mu, lam, vol) -> float:
    """sum vol psi(J x).  simkit ``macklin_mueller_neo_hookean_energy_x`` (:484-509)."""
    m = _bind(J, mu, lam, vol, MATERIALS["macklin-mueller-neo-hookean"])
    x = _dev(X).reshape(-1)
    ws = m.workspace(SKG_FP64)
    e = ctypes.c_double()
    check(_lib.load().skg_snh_energy_x(ctypes.byref(m.c), _ptr(x), ctypes.byref(e), _ptr(ws), _stream_ptr()))
    return float(e.value)


def macklin_mueller_neo_hookean_gradient_x(X, J, mu, lam, vol):
    """J^T vec(vol P), (3n, 1).  simkit ``macklin_mueller_neo_hookean_gradient_x`` (:512-538)."""
    m = _bind(J, mu, lam, vol, MATERIALS["macklin-mueller-neo-hookean"])
    x = _dev(X).reshape(-1)
    ws = m.workspace(SKG_FP64)
    g = torch.empty(3 * m.n, dtype=torch.float64, device="cuda")
    check(_lib.load().skg_snh_gradient_x(ctypes.byref(m.c), _ptr(x), _ptr(g), _ptr(ws), _stream_ptr()))
    return _out(g.reshape(-1, 1), X)


def macklin_mueller_neo_hookean_hessian_x(X, J, mu, lam, vol, psd: bool = True, precision: str = "fp64"):
    """J^T blockdiag(psd(vol He)) J.  simkit ``macklin_mueller_neo_hookean_hessian_x`` (:541-574)."""
    m = _bind(J, mu, lam, vol, MATERIALS["macklin-mueller-neo-hookean"])
    B = BlockMatrix(m, assemble_hessian_blocks(m, X, precision=precision, psd=psd))
    return B if isinstance(X, torch.Tensor) else B.to_scipy()


def macklin_mueller_neo_hookean_energy(X, T, mu, lam, U: Optional[np.ndarray] = None) -> float:
    """simkit ``macklin_mueller_neo_hookean_energy`` (:689-714)."""
    return macklin_mueller_neo_hookean_energy_x(X if U is None else U, deformation_jacobian(X, T), mu, lam,
                                                volume(X, T))


def macklin_mueller_neo_hookean_gradient(X, T, mu, lam, U: Optional[np.ndarray] = None):
    """simkit ``macklin_mueller_neo_hookean_gradient`` (:717-742)."""
    return macklin_mueller_neo_hookean_gradient_x(X if U is None else U, deformation_jacobian(X, T), mu, lam,
                                                  volume(X, T))


def macklin_mueller_neo_hookean_hessian(X, T, mu, lam, U: Optional[np.ndarray] = None, psd: bool = True):
    """simkit ``macklin_mueller_neo_hookean_hessian`` (:745-773)."""
    return macklin_mueller_neo_hookean_hessian_x(X if U is None else U, deformation_jacobian(X, T), mu, lam,
                                                 volume(X, T), psd=psd)


# --------------------------------------------------------------------------- #
# corotational energies: simkit/energies/arap.py, simkit/energies/fcr.py       #
# --------------------------------------------------------------------------- #
def _energy_x(X, J, mu, lam, vol, material) -> float:
    m = _bind(J, mu, lam, vol, material)
    x = _dev(X).reshape(-1)
    ws = m.workspace(SKG_FP64)
    e = ctypes.c_double()
    check(_lib.load().skg_snh_energy_x(ctypes.byref(m.c), _ptr(x), ctypes.byref(e), _ptr(ws), _stream_ptr()))
    return float(e.value)


def _gradient_x(X, J, mu, lam, vol, material):
    m = _bind(J, mu, lam, vol, material)
    x = _dev(X).reshape(-1)
    ws = m.workspace(SKG_FP64)
    g = torch.empty(3 * m.n, dtype=torch.float64, device="cuda")
    check(_lib.load().skg_snh_gradient_x(ctypes.byref(m.c), _ptr(x), _ptr(g), _ptr(ws), _stream_ptr()))
    return _out(g.reshape(-1, 1), X)


def _hessian_x(X, J, mu, lam, vol, material, psd, precision):
    m = _bind(J, mu, lam, vol, material)
    B = BlockMatrix(m, assemble_hessian_blocks(m, X, precision=precision, psd=psd))
    return B if isinstance(X, torch.Tensor) else B.to_scipy()


# displacement tier: F = J u + Jx_bar (simkit's *_u functions)
def _jx_bar(Jx_bar, m: TetMesh):
    f = _dev(Jx_bar).reshape(-1)
    if f.numel() != 9 * m.t:
        raise ValueError(f"Jx_bar needs 9 values per tet ({9 * m.t}), got {f.numel()}")
    return f


def _energy_u(u, J, Jx_bar, mu, lam, vol, material) -> float:
    m = _bind(J, mu, lam, vol, material)
    ud = _dev(u).reshape(-1)
    f = _jx_bar(Jx_bar, m)
    ws = m.workspace(SKG_FP64)
    e = ctypes.c_double()
    check(_lib.load().skg_snh_energy_u(ctypes.byref(m.c), _ptr(ud), _ptr(f), ctypes.byref(e), _ptr(ws),
                                       _stream_ptr()))
    return float(e.value)


def _gradient_u(u, J, Jx_bar, mu, lam, vol, material):
    m = _bind(J, mu, lam, vol, material)
    ud = _dev(u).reshape(-1)
    f = _jx_bar(Jx_bar, m)
    ws = m.workspace(SKG_FP64)
    g = torch.empty(3 * m.n, dtype=torch.float64, device="cuda")
    check(_lib.load().skg_snh_gradient_u(ctypes.byref(m.c), _ptr(ud), _ptr(f), _ptr(g), _ptr(ws), _stream_ptr()))
    return _out(g.reshape(-1, 1), u)


def _hessian_u(u, J, Jx_bar, mu, lam, vol, material, psd, precision):
    m = _bind(J, mu, lam, vol, material)
    ud = _dev(u).reshape(-1)
    f = _jx_bar(Jx_bar, m)
    prec = _PREC[precision]
    ws = m.workspace(prec)
    dt = torch.float64 if prec == SKG_FP64 else torch.float32
    val = torch.empty(9 * m.nb, dtype=dt, device="cuda")
    v64, v32 = (val, None) if prec == SKG_FP64 else (None, val)
    check(_lib.load().skg_snh_hessian_u(ctypes.byref(m.c), _ptr(ud), _ptr(f), prec, int(psd), _ptr(v64), _ptr(v32),
                                        _ptr(ws), _stream_ptr()))
    B = BlockMatrix(m, val)
    return B if isinstance(u, torch.Tensor) else B.to_scipy()


def stable_neo_hookean_energy_u(u, J, Jx_bar, mu, lam, vol) -> float:
    """sum vol psi(J u + Jx_bar).  simkit ``stable_neo_hookean_energy_u`` (snh.py:544-576)."""
    return _energy_u(u, J, Jx_bar, mu, lam, vol, MATERIALS["stable-neo-hookean"])


def stable_neo_hookean_gradient_u(u, J, Jx_bar, mu, lam, vol):
    """J^T vec(vol P(J u + Jx_bar)), (3n, 1).  simkit ``stable_neo_hookean_gradient_u`` (snh.py:579-611)."""
    return _gradient_u(u, J, Jx_bar, mu, lam, vol, MATERIALS["stable-neo-hookean"])


def stable_neo_hookean_hessian_u(u, J, Jx_bar, mu, lam, vol, psd: bool = True, precision: str = "fp64"):
    """J^T blockdiag(psd(vol He)) J at F = J u + Jx_bar.  simkit ``stable_neo_hookean_hessian_u``
    (snh.py:614-648)."""
    return _hessian_u(u, J, Jx_bar, mu, lam, vol, MATERIALS["stable-neo-hookean"], psd, precision)


def macklin_mueller_neo_hookean_energy_u(u, J, Jx_bar, mu, lam, vol) -> float:
    """simkit ``macklin_mueller_neo_hookean_energy_u`` (:579-611)."""
    return _energy_u(u, J, Jx_bar, mu, lam, vol, MATERIALS["macklin-mueller-neo-hookean"])


def macklin_mueller_neo_hookean_gradient_u(u, J, Jx_bar, mu, lam, vol):
    """simkit ``macklin_mueller_neo_hookean_gradient_u`` (:614-646)."""
    return _gradient_u(u, J, Jx_bar, mu, lam, vol, MATERIALS["macklin-mueller-neo-hookean"])


def macklin_mueller_neo_hookean_hessian_u(u, J, Jx_bar, mu, lam, vol, psd: bool = True, precision: str = "fp64"):
    """simkit ``macklin_mueller_neo_hookean_hessian_u`` (:649-683)."""
    return _hessian_u(u, J, Jx_bar, mu, lam, vol, MATERIALS["macklin-mueller-neo-hookean"], psd, precision)


def _no_lam(mu):
    """ARAP has no volume term; the kernels take a lam array and ignore it."""
    return mu


def arap_energy_element_F(F, mu, precision: str = "fp64"):
    """psi = mu/2 |F - R|^2 per element, (t, 1).  simkit ``arap_energy_element_F`` (arap.py:71-91)."""
    return _elem("skg_arap_energy_element_F", F, mu, _no_lam(mu), lambda t, d: (t, 1), precision, "ARAP")


def arap_gradient_element_F(F, mu, precision: str = "fp64"):
    """P = mu (F - R), (t, d, d).  simkit ``arap_gradient_element_F`` (arap.py:94-114)."""
    return _elem("skg_arap_gradient_element_F", F, mu, _no_lam(mu), lambda t, d: (t, d, d), precision, "ARAP")


def arap_hessian_element_F(F, mu, precision: str = "fp64"):
    """mu (I - dR/dF), (t, d*d, d*d), not projected.  simkit ``arap_hessian_element_F`` (arap.py:117-145)."""
    return _elem("skg_arap_hessian_element_F", F, mu, _no_lam(mu), lambda t, d: (t, d * d, d * d), precision, "ARAP")


def arap_energy_x(X, J, mu, vol) -> float:
    """sum vol psi(J x).  simkit ``arap_energy_x`` (arap.py:242-265)."""
    return _energy_x(X, J, mu, _no_lam(mu), vol, MATERIALS["arap"])


def arap_gradient_x(X, J, mu, vol):
    """J^T vec(vol P), (3n, 1).  simkit ``arap_gradient_x`` (arap.py:268-292)."""
    return _gradient_x(X, J, mu, _no_lam(mu), vol, MATERIALS["arap"])


def arap_hessian_x(X, J, mu, vol, psd: bool = True, precision: str = "fp64"):
    """J^T blockdiag(psd(vol He)) J.  simkit ``arap_hessian_x`` (arap.py:295-325)."""
    return _hessian_x(X, J, mu, _no_lam(mu), vol, MATERIALS["arap"], psd, precision)


def arap_energy(X, T, mu, U: Optional[np.ndarray] = None) -> float:
    """simkit ``arap_energy`` (arap.py:505-529)."""
    return arap_energy_x(X if U is None else U, deformation_jacobian(X, T), mu, volume(X, T))


def arap_gradient(X, T, mu, U: Optional[np.ndarray] = None):
    """simkit ``arap_gradient`` (arap.py:532-555)."""
    return arap_gradient_x(X if U is None else U, deformation_jacobian(X, T), mu, volume(X, T))


def arap_hessian(X, T, mu, U: Optional[np.ndarray] = None, psd: bool = True):
    """simkit ``arap_hessian`` (arap.py:558-583)."""
    return arap_hessian_x(X if U is None else U, deformation_jacobian(X, T), mu, volume(X, T), psd=psd)


def arap_energy_u(u, J, Jx_bar, mu, vol) -> float:
    """simkit ``arap_energy_u`` (arap.py:331-360)."""
    return _energy_u(u, J, Jx_bar, mu, _no_lam(mu), vol, MATERIALS["arap"])


def arap_gradient_u(u, J, Jx_bar, mu, vol):
    """simkit ``arap_gradient_u`` (arap.py:363-389)."""
    return _gradient_u(u, J, Jx_bar, mu, _no_lam(mu), vol, MATERIALS["arap"])


def arap_hessian_u(u, J, Jx_bar, mu, vol, psd: bool = True, precision: str = "fp64"):
    """simkit ``arap_hessian_u`` (arap.py:392-424)."""
    return _hessian_u(u, J, Jx_bar, mu, _no_lam(mu), vol, MATERIALS["arap"], psd, precision)


def fcr_energy_element_F(F, mu, lam, precision: str = "fp64"):
    """psi = mu |F - R|^2 + lam/2 (J - 1)^2 per element, (t, 1).  simkit ``fcr_energy_element_F`` (fcr.py:41-62)."""
    return _elem("skg_fcr_energy_element_F", F, mu, lam, lambda t, d: (t, 1), precision, "FCR")


def fcr_gradient_element_F(F, mu, lam, precision: str = "fp64"):
    """P = 2 mu (F - R) + lam (J - 1) cof F, (t, d, d).  simkit ``fcr_gradient_element_F`` (fcr.py:65-125)."""
    return _elem("skg_fcr_gradient_element_F", F, mu, lam, lambda t, d: (t, d, d), precision, "FCR")


def fcr_hessian_element_F(F, mu, lam, precision: str = "fp64"):
    """(t, d*d, d*d), not projected.  simkit ``fcr_hessian_element_F`` (fcr.py:128-302)."""
    return _elem("skg_fcr_hessian_element_F", F, mu, lam, lambda t, d: (t, d * d, d * d), precision, "FCR")


def fcr_energy_x(X, J, mu, lam, vol) -> float:
    """sum vol psi(J x).  simkit ``fcr_energy_x`` (fcr.py:308-333)."""
    return _energy_x(X, J, mu, lam, vol, MATERIALS["fcr"])


def fcr_gradient_x(X, J, mu, lam, vol):
    """J^T vec(vol P), (3n, 1).  simkit ``fcr_gradient_x`` (fcr.py:336-362)."""
    return _gradient_x(X, J, mu, lam, vol, MATERIALS["fcr"])


def fcr_hessian_x(X, J, mu, lam, vol, psd: bool = True, precision: str = "fp64"):
    """J^T blockdiag(psd(vol He)) J.  simkit ``fcr_hessian_x`` (fcr.py:365-397)."""
    return _hessian_x(X, J, mu, lam, vol, MATERIALS["fcr"], psd, precision)


def fcr_energy_u(u, J, Jx_bar, mu, lam, vol) -> float:
    """simkit ``fcr_energy_u`` (fcr.py:403-434)."""
    return _energy_u(u, J, Jx_bar, mu, lam, vol, MATERIALS["fcr"])


def fcr_gradient_u(u, J, Jx_bar, mu, lam, vol):
    """simkit ``fcr_gradient_u`` (fcr.py:437-465)."""
    return _gradient_u(u, J, Jx_bar, mu, lam, vol, MATERIALS["fcr"])


def fcr_hessian_u(u, J, Jx_bar, mu, lam, vol, psd: bool = True, precision: str = "fp64"):
    """simkit ``fcr_hessian_u`` (fcr.py:468-502)."""
    return _hessian_u(u, J, Jx_bar, mu, lam, vol, MATERIALS["fcr"], psd, precision)


def fcr_energy(X, T, mu, lam, U: Optional[np.ndarray] = None) -> float:
    """simkit ``fcr_energy`` (fcr.py:508-533)."""
    return fcr_energy_x(X if U is None else U, deformation_jacobian(X, T), mu, lam, volume(X, T))


def fcr_gradient(X, T, mu, lam, U: Optional[np.ndarray] = None):
    """simkit ``fcr_gradient`` (fcr.py:536-561)."""
    return fcr_gradient_x(X if U is None else U, deformation_jacobian(X, T), mu, lam, volume(X, T))


def fcr_hessian(X, T, mu, lam, U: Optional[np.ndarray] = None, psd: bool = True):
    """simkit ``fcr_hessian`` (fcr.py:564-591)."""
    return fcr_hessian_x(X if U is None else U, deformation_jacobian(X, T), mu, lam, volume(X, T), psd=psd)


# --------------------------------------------------------------------------- #
# linear elasticity: simkit/energies/linear_elasticity.py                      #
# --------------------------------------------------------------------------- #
_LE = "Linear elasticity"


def linear_elasticity_energy_element_F(F, mu, lam, precision: str = "fp64"):
    """psi = mu |eps|^2 + lam/2 tr(eps)^2, eps = sym(F) - I, (t, 1).  simkit
    ``linear_elasticity_energy_element_F`` (linear_elasticity.py:43-70)."""
    return _elem("skg_le_energy_element_F", F, mu, lam, lambda t, d: (t, 1), precision, _LE)


def linear_elasticity_gradient_element_F(F, mu, lam, precision: str = "fp64"):
    """P = mu (F + F^T - 2 I) + lam tr(F - I) I, (t, d, d).  simkit ``linear_elasticity_gradient_element_F`` (:73-100)."""
    return _elem("skg_le_gradient_element_F", F, mu, lam, lambda t, d: (t, d, d), precision, _LE)


def linear_elasticity_hessian_element_F(F, mu, lam, precision: str = "fp64"):
    """mu (I + T) + lam vec(I) vec(I)^T, (t, d*d, d*d).  simkit ``linear_elasticity_hessian_element_F`` (:103-136)."""
    return _elem("skg_le_hessian_element_F", F, mu, lam, lambda t, d: (t, d * d, d * d), precision, _LE)


def linear_elasticity_energy_x(X, J, mu, lam, vol) -> float:
    """simkit ``linear_elasticity_energy_x`` (:142-167)."""
    return _energy_x(X, J, mu, lam, vol, MATERIALS["linear-elasticity"])


def linear_elasticity_gradient_x(X, J, mu, lam, vol):
    """simkit ``linear_elasticity_gradient_x`` (:170-196)."""
    return _gradient_x(X, J, mu, lam, vol, MATERIALS["linear-elasticity"])


def linear_elasticity_hessian_x(X, J, mu, lam, vol, psd: bool = True, precision: str = "fp64"):
    """J^T blockdiag(vol He) J; ``psd`` is accepted and has no effect, as in simkit
    ``linear_elasticity_hessian_x`` (:199-230): the Hessian is constant and PSD."""
    return _hessian_x(X, J, mu, lam, vol, MATERIALS["linear-elasticity"], psd, precision)


def linear_elasticity_energy_u(u, J, Jx_bar, mu, lam, vol) -> float:
    """simkit ``linear_elasticity_energy_u`` (:236-267)."""
    return _energy_u(u, J, Jx_bar, mu, lam, vol, MATERIALS["linear-elasticity"])


def linear_elasticity_gradient_u(u, J, Jx_bar, mu, lam, vol):
    """simkit ``linear_elasticity_gradient_u`` (:270-298)."""
    return _gradient_u(u, J, Jx_bar, mu, lam, vol, MATERIALS["linear-elasticity"])


def linear_elasticity_hessian_u(u, J, Jx_bar, mu, lam, vol, psd: bool = True, precision: str = "fp64"):
    """simkit ``linear_elasticity_hessian_u`` (:301-333); ``psd`` has no effect."""
    return _hessian_u(u, J, Jx_bar, mu, lam, vol, MATERIALS["linear-elasticity"], psd, precision)


def linear_elasticity_energy(X, T, mu, lam, U: Optional[np.ndarray] = None) -> float:
    """simkit ``linear_elasticity_energy`` (:339-364)."""
    return linear_elasticity_energy_x(X if U is None else U, deformation_jacobian(X, T), mu, lam, volume(X, T))


def linear_elasticity_gradient(X, T, mu, lam, U: Optional[np.ndarray] = None):
    """simkit ``linear_elasticity_gradient`` (:367-392)."""
    return linear_elasticity_gradient_x(X if U is None else U, deformation_jacobian(X, T), mu, lam, volume(X, T))


def linear_elasticity_hessian(X, T, mu, lam, U: Optional[np.ndarray] = None, psd: bool = True):
    """simkit ``linear_elasticity_hessian`` (:395-423)."""
    return linear_elasticity_hessian_x(X if U is None else U, deformation_jacobian(X, T), mu, lam, volume(X, T),
                                       psd=psd)


# --------------------------------------------------------------------------- #
# contact springs: simkit/energies/contact_springs_plane.py:44-200             #
# --------------------------------------------------------------------------- #
def _contact(X, k, p, n, M):
    Xd = _dev(X)
    nv = Xd.numel() // 3
    if Xd.numel() != 3 * nv or (X.ndim == 2 and X.shape[1] != 3):
        raise ValueError("the GPU contact springs support 3D positions")
    arr, _ = _lib.contact_planes([(k, np.asarray(p).reshape(-1)[:3], np.asarray(n, dtype=np.float64).reshape(3))])
    # simkit uses n as given (no normalisation)
    arr[0].n[:] = list(np.asarray(n, dtype=np.float64).reshape(3))
    m = None
    if M is not None:
        diag = M.diagonal() if sps.issparse(M) else np.diagonal(np.asarray(M))
        m = _dev(np.asarray(diag, dtype=np.float64).reshape(-1))
    return Xd.reshape(-1), nv, arr, m


def _contact_inds(under):
    idx = np.nonzero(under.cpu().numpy())[0]
    return idx[:, None] if idx.size else None


def contact_springs_plane_energy(X, k: float, p, n, M=None, return_contact_inds: bool = False):
    """simkit ``contact_springs_plane_energy`` (contact_springs_plane.py:44-86): sum over vertices
    below the plane of k m (n.(x - p))^2 / 2, m the diagonal of M (default identity)."""
    Xd, nv, arr, m = _contact(X, k, p, n, M)
    ev = torch.empty(nv, dtype=torch.float64, device="cuda")
    under = torch.empty(nv, dtype=torch.uint8, device="cuda")
    check(_lib.load().skg_contact_plane_terms(_ptr(Xd), nv, arr, _ptr(m), _ptr(ev), None, None, _ptr(under),
                                              _stream_ptr()))
    e = float(ev.cpu().numpy().sum())
    return (e, _contact_inds(under)) if return_contact_inds else e


def contact_springs_plane_gradient(X, k: float, p, n, M=None, return_contact_inds: bool = False):
    """simkit ``contact_springs_plane_gradient`` (:87-130), (3n, 1)."""
    Xd, nv, arr, m = _contact(X, k, p, n, M)
    g = torch.empty(3 * nv, dtype=torch.float64, device="cuda")
    under = torch.empty(nv, dtype=torch.uint8, device="cuda")
    check(_lib.load().skg_contact_plane_terms(_ptr(Xd), nv, arr, _ptr(m), None, _ptr(g), None, _ptr(under),
                                              _stream_ptr()))
    out = _out(g.reshape(-1, 1), X)
    return (out, _contact_inds(under)) if return_contact_inds else out


def contact_springs_plane_hessian(X, k: float, p, n, M=None, return_contact_inds: bool = False):
    """simkit ``contact_springs_plane_hessian`` (:131-200): block diagonal k m n n^T on the
    vertices below the plane, scipy csc (3n x 3n)."""
    Xd, nv, arr, m = _contact(X, k, p, n, M)
    h = torch.empty(9 * nv, dtype=torch.float64, device="cuda")
    under = torch.empty(nv, dtype=torch.uint8, device="cuda")
    check(_lib.load().skg_contact_plane_terms(_ptr(Xd), nv, arr, _ptr(m), None, None, _ptr(h), _ptr(under),
                                              _stream_ptr()))
    hb = h.cpu().numpy().reshape(nv, 3, 3)
    idx = np.nonzero(under.cpu().numpy())[0]
    rows = (3 * idx[:, None, None] + np.arange(3)[None, :, None]).repeat(3, 2)
    cols = (3 * idx[:, None, None] + np.arange(3)[None, None, :]).repeat(3, 1)
    H = sps.csc_matrix((hb[idx].ravel(), (rows.ravel(), cols.ravel())), shape=(3 * nv, 3 * nv))
    return (H, _contact_inds(under)) if return_contact_inds else H


# --------------------------------------------------------------------------- #
# material dispatch: simkit/energies/elastic.py                               #
# --------------------------------------------------------------------------- #
_PREFIX = {"macklin-mueller-neo-hookean": "macklin_mueller_neo_hookean", "arap": "arap", "fcr": "fcr",
           "linear-elasticity": "linear_elasticity"}


def _material(material, lam_args):
    """(function-name prefix, lam-carrying positional args) of ``material``; ARAP's functions
    take no lam (simkit/energies/elastic.py passes lam to every material but ARAP)."""
    if material in _PREFIX:
        return _PREFIX[material], (() if material == "arap" else lam_args)
    raise ValueError("Unknown material type: " + str(material))


def elastic_energy_element_F(F, mu, lam, material: str):
    """simkit ``elastic_energy_element_F`` (elastic.py:86-116)."""
    pre, la = _material(material, (lam,))
    return globals()[pre + "_energy_element_F"](F, mu, *la)


def elastic_gradient_element_F(F, mu, lam, material: str):
    """simkit ``elastic_gradient_element_F`` (elastic.py:396-426)."""
    pre, la = _material(material, (lam,))
    return globals()[pre + "_gradient_element_F"](F, mu, *la)


def elastic_hessian_element_F(F, mu, lam, material: str, psd: bool = True):
    """simkit ``elastic_hessian_element_F`` (elastic.py:632-668): unweighted blocks, projected if psd."""
    pre, la = _material(material, (lam,))
    Q = globals()[pre + "_hessian_element_F"](F, mu, *la)
    return psd_project(Q) if psd else Q


def elastic_energy_x(X, J, mu, lam, vol, material: str) -> float:
    """simkit ``elastic_energy_x`` (elastic.py:119-148)."""
    pre, la = _material(material, (lam,))
    return globals()[pre + "_energy_x"](X, J, mu, *la, vol)


def elastic_gradient_x(X, J, mu, lam, vol, material: str):
    """simkit ``elastic_gradient_x`` (elastic.py:429-459)."""
    pre, la = _material(material, (lam,))
    return globals()[pre + "_gradient_x"](X, J, mu, *la, vol)


def elastic_hessian_x(X, J, mu, lam, vol, material: str, psd: bool = True):
    """simkit ``elastic_hessian_x`` (elastic.py:671-705)."""
    pre, la = _material(material, (lam,))
    return globals()[pre + "_hessian_x"](X, J, mu, *la, vol, psd=psd)


def elastic_energy_u(u, J, Jx_bar, mu, lam, vol, material: str) -> float:
    """simkit ``elastic_energy_u`` (elastic.py:151-188)."""
    pre, la = _material(material, (lam,))
    return globals()[pre + "_energy_u"](u, J, Jx_bar, mu, *la, vol)


def elastic_gradient_u(u, J, Jx_bar, mu, lam, vol, material: str):
    """simkit ``elastic_gradient_u`` (elastic.py:462-497)."""
    pre, la = _material(material, (lam,))
    return globals()[pre + "_gradient_u"](u, J, Jx_bar, mu, *la, vol)


def elastic_hessian_u(u, J, Jx_bar, mu, lam, vol, material: str, psd: bool = True):
    """simkit ``elastic_hessian_u`` (elastic.py:708-746)."""
    pre, la = _material(material, (lam,))
    return globals()[pre + "_hessian_u"](u, J, Jx_bar, mu, *la, vol, psd=psd)


def elastic_energy(X, T, mu, lam, material: str, U: Optional[np.ndarray] = None) -> float:
    """simkit ``elastic_energy`` (elastic.py:360-393)."""
    pre, la = _material(material, (lam,))
    return globals()[pre + "_energy"](X, T, mu, *la, U)


def elastic_gradient(X, T, mu, lam, material: str, U: Optional[np.ndarray] = None):
    """simkit ``elastic_gradient`` (elastic.py:596-629)."""
    pre, la = _material(material, (lam,))
    return globals()[pre + "_gradient"](X, T, mu, *la, U)


def elastic_hessian(X, T, mu, lam, material: str, U: Optional[np.ndarray] = None, psd: bool = True):
    """simkit ``elastic_hessian`` (elastic.py:849-882)."""
    pre, la = _material(material, (lam,))
    return globals()[pre + "_hessian"](X, T, mu, *la, U, psd=psd)


# --------------------------------------------------------------------------- #
# linear solve standing in for spsolve (simkit/solvers/newton.py:52)           #
# --------------------------------------------------------------------------- #
def _diagonal_of(M, N: int):
    """The diagonal (N,) of a diagonal matrix M (scipy sparse or dense, N x N), else None."""
    if sps.issparse(M):
        if M.shape != (N, N):
            return None
        d = np.asarray(M.diagonal(), dtype=np.float64)
        C = sps.coo_matrix(M)
        if np.any((C.row != C.col) & (C.data != 0)):
            return None
        return d
    if isinstance(M, torch.Tensor):
        M = M.detach().cpu().numpy()
    A = np.asarray(M, dtype=np.float64)
    if A.shape != (N, N):
        return None
    d = np.diagonal(A).copy()
    if np.count_nonzero(A - np.diag(d)):
        return None
    return d


class _BlockPlan:
    """The 3x3-block CSR pattern (every diagonal block present, rows padded to a multiple of 3 with
    the identity) of a scalar CSR pattern, and the scatter of the scalar values into the solver's
    entry-major block values: val[dst] = data (padding diagonal entries at pad_dst get 1)."""

    def __init__(self, indptr, indices, n):
        self.indptr, self.indices, self.n = indptr.copy(), indices.copy(), n
        N = n + (-n) % 3
        nbr = N // 3
        rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(indptr))
        cols = indices.astype(np.int64)
        br, bc = rows // 3, cols // 3
        keys = np.unique(np.concatenate([br * nbr + bc, np.arange(nbr, dtype=np.int64) * (nbr + 1)]))
        krow = keys // nbr
        rowptr = np.zeros(nbr + 1, np.int64)
        rowptr[1:] = np.cumsum(np.bincount(krow, minlength=nbr))
        K = np.diff(rowptr)

        def dst_of(r, c):
            slot = np.searchsorted(keys, (r // 3) * nbr + c // 3)
            v = r // 3
            return 9 * rowptr[v] + (3 * (r % 3) + c % 3) * K[v] + (slot - rowptr[v])

        self.dst = dst_of(rows, cols)
        pad = np.arange(n, N, dtype=np.int64)
        self.pad_dst = dst_of(pad, pad)
        self.nbr, self.N, self.nvals = nbr, N, 9 * keys.size
        self.rowptr = rowptr.astype(np.int32)
        self.col = (keys % nbr).astype(np.int32)

    def matches(self, A) -> bool:
        return (A.shape[0] == self.n and A.indptr.size == self.indptr.size and A.indices.size == self.indices.size
                and np.array_equal(A.indptr, self.indptr) and np.array_equal(A.indices, self.indices))

    def values(self, data) -> np.ndarray:
        val = np.zeros(self.nvals)
        if self.has_duplicates:   # a CSR matrix not in canonical form: repeated entries add
            np.add.at(val, self.dst, data)
        else:
            val[self.dst] = data
        val[self.pad_dst] = 1.0
        return val

    @property
    def has_duplicates(self) -> bool:
        """Whether a row repeats a column (or lists its columns unsorted: then summed the slow way)."""
        if not hasattr(self, "_dup"):
            d = np.diff(self.indices.astype(np.int64)) > 0
            starts = self.indptr[1:-1].astype(np.int64)
            d[starts[(starts > 0) & (starts < self.indices.size)] - 1] = True   # steps into the next row
            self._dup = not bool(d.all())
        return self._dup


_PLANS: dict = {}   # block plans by scalar pattern size (a Newton loop reuses one pattern)


def _block_plan(A) -> _BlockPlan:
    key = (A.shape[0], A.nnz)
    plan = _PLANS.get(key)
    if plan is None or not plan.matches(A):
        plan = _BlockPlan(A.indptr, A.indices, A.shape[0])
        if len(_PLANS) >= 8:
            _PLANS.pop(next(iter(_PLANS)))
        _PLANS[key] = plan
    if not hasattr(plan, "rowptr_d"):
        plan.rowptr_d = torch.from_numpy(plan.rowptr).cuda()
        plan.col_d = torch.from_numpy(plan.col).cuda()
    return plan


def _pcg64(nbr, rowptr_d, col_d, val_d, b_d, rtol, max_iter):
    lib = _lib.load()
    x_d = torch.empty(3 * nbr, dtype=torch.float64, device=val_d.device)
    ws = torch.empty(int(lib.skg_pcg_workspace_size(nbr)), dtype=torch.uint8, device=val_d.device)
    iters = ctypes.c_int32()
    check(lib.skg_pcg_bsr64(nbr, _ptr(rowptr_d), _ptr(col_d), _ptr(val_d), _ptr(b_d), _ptr(x_d), rtol, max_iter,
                            ctypes.byref(iters), _ptr(ws), _stream_ptr()))
    return x_d


def solve_sparse(A, b, rtol: float = 1e-12, max_iter: int = 20000):
    """x = A^{-1} b for symmetric positive definite A by FP64 block-Jacobi PCG on the GPU (the
    replacement of simkit's ``spsolve`` in solvers/newton.py:52).

    A may be a scipy sparse matrix, a dense array or a ``BlockMatrix``.  A ``BlockMatrix`` is solved
    where it lives (the mesh's block pattern and the device values).  A scipy matrix goes through a
    block plan cached by its sparsity pattern, so the repeated solves of a Newton loop copy only the
    values (one scatter on the host, one host-to-device copy).
    """
    torch_b = isinstance(b, torch.Tensor)
    if isinstance(A, BlockMatrix):
        m = A.mesh
        b_d = (b.detach().to(m.device, torch.float64) if torch_b
               else torch.from_numpy(np.asarray(b, dtype=np.float64)).to(m.device)).reshape(-1).contiguous()
        x = _pcg64(m.n, m.rowptr, m.col, A.val.double().contiguous(), b_d, rtol, max_iter).reshape(-1, 1)
        return x if torch_b else x.cpu().numpy()
    if not sps.issparse(A):
        A = sps.csr_matrix(np.asarray(A, dtype=np.float64))
    A = sps.csr_matrix(A, dtype=np.float64)
    n = A.shape[0]
    plan = _block_plan(A)
    bb = np.zeros(plan.N)
    bb[:n] = b.detach().cpu().numpy().reshape(-1) if torch_b else np.asarray(b, dtype=np.float64).reshape(-1)
    val_d = torch.from_numpy(plan.values(A.data)).cuda()
    x = _pcg64(plan.nbr, plan.rowptr_d, plan.col_d, val_d, torch.from_numpy(bb).cuda(), rtol, max_iter)
    x = x[:n].reshape(-1, 1)
    return x if torch_b else x.cpu().numpy()


# --------------------------------------------------------------------------- #
# line search / Newton / backward Euler                                       #
# --------------------------------------------------------------------------- #
def backtracking_line_search(f, x0, g, dx, alpha: float = 0.01, beta: float = 0.5, max_iter: int = 100,
                             threshold: float = 1e-12):
    """simkit ``backtracking_line_search`` (backtracking_line_search.py:8-67), same contract:
    returns (t, x0 + t dx, f) for the first t = beta^k passing Armijo, else (0, x0, f(x0))."""
    assert alpha > 0 and alpha <= 0.5
    assert beta > 0 and beta < 1
    assert np.ndim(x0) == np.ndim(dx)
    t = 1.0
    fx0 = f(x0)
    slope = g.T @ dx
    for _ in range(max_iter):
        x = x0 + t * dx
        fx = f(x)
        if fx <= fx0 + alpha * t * slope + threshold:
            return t, x, fx
        t = beta * t
    return 0.0, x0, fx0


def newton_solver(x0, energy_func, gradient_func, hessian_func, tolerance=1e-6, max_iter=1, do_line_search=True,
                  return_info=False):
    """simkit ``newton_solver`` (solvers/newton.py:7-75) with the linear solve on the GPU.

    ``spsolve(H, -g)`` (newton.py:52) is replaced by block-Jacobi PCG to a
    relative residual of 1e-12 in FP64.
    """
    x = x0.copy() if not isinstance(x0, torch.Tensor) else x0.clone()
    if return_info:
        info = {"g": [], "dx": [], "alphas": [], "iters": -1}
    for i in range(max_iter):
        g = gradient_func(x)
        H = hessian_func(x)
        dx = solve_sparse(H, -g).reshape(-1, 1)
        if do_line_search:
            alpha, _, _ = backtracking_line_search(energy_func, x, g, dx)
        else:
            alpha = 1.0
        x += alpha * dx
        if return_info:
            info["g"].append(g)
            info["dx"].append(dx)
            info["alphas"].append(alpha)
            info["iters"] = i
        nrm = float(torch.linalg.norm(alpha * dx)) if isinstance(dx, torch.Tensor) else float(np.linalg.norm(alpha * dx))
        if nrm < tolerance:
            break
    if return_info:
        return x, info
    return x


class ElasticPotential:
    """V(x) = sum_e vol_e psi(F_e(x)) - f_ext . x for one tet mesh, with simkit's closure signatures:
    ``energy(x) -> float``, ``gradient(x) -> (3n, 1)``, ``hessian(x) -> sparse (3n, 3n)`` (PSD-projected
    element blocks, as simkit's ``*_hessian_x`` default), x the (3n, 1) positions.

    Handed to ``backward_euler`` as ``(pot.energy, pot.gradient, pot.hessian)`` with a lumped
    (diagonal) mass matrix, the whole Newton solve runs on the device (``BESolver`` with simkit's
    stop rule ``||alpha dx|| < tolerance``, at most ``max_iter`` iterations, FP64 with the linear
    solves to 1e-12); any other closures take the closure path, as in simkit.
    """

    def __init__(self, X, T, mu, lam, material: str = "stable-neo-hookean", f_ext=None):
        self.X = np.asarray(X, dtype=np.float64)
        self.T = np.asarray(T)
        self.mu = np.asarray(mu, dtype=np.float64).reshape(-1)
        self.lam = np.asarray(lam, dtype=np.float64).reshape(-1)
        if material not in MATERIALS:
            raise ValueError("Unknown material type: " + str(material))
        self.material = material
        self.J = deformation_jacobian(self.X, self.T)
        self.vol = volume(self.X, self.T)
        n3 = self.X.size
        self.f_ext = np.zeros((n3, 1)) if f_ext is None else np.asarray(f_ext, dtype=np.float64).reshape(n3, 1)
        self._steppers = {}

    def _args(self):
        return self.J, self.mu, self.lam, self.vol, MATERIALS[self.material]

    def energy(self, x) -> float:
        J, mu, lam, vol, code = self._args()
        return _energy_x(x, J, mu, lam, vol, code) - float((self.f_ext.T @ np.asarray(x).reshape(-1, 1)).item())

    def gradient(self, x):
        J, mu, lam, vol, code = self._args()
        return _gradient_x(x, J, mu, lam, vol, code) - self.f_ext

    def hessian(self, x):
        J, mu, lam, vol, code = self._args()
        return _hessian_x(x, J, mu, lam, vol, code, True, "fp64")

    def stepper(self, h: float, mass, integrator: str = "be"):
        """The device stepper for step h, per-vertex masses and integrator ('be' or 'bdf2'), cached."""
        from .solver import BESolver
        key = (float(h), np.asarray(mass).tobytes(), integrator)
        if key not in self._steppers:
            self._steppers[key] = BESolver(self.X, self.T, self.mu, self.lam, dt=float(h), precision="fp64",
                                           pcg_rtol=1e-12, pcg_max_iter=20000, material=self.material,
                                           mass=mass, f_ext=self.f_ext, integrator=integrator)
        return self._steppers[key]

    def _device_step(self, integrator, M, h, tolerance, max_iter, do_line_search, xs, return_info=False):
        """simkit's Newton contract on the device, or None when M is not lumped.  With return_info,
        (x_next, info): simkit's newton_solver info (newton.py:43-67: per-iteration gradient 'g' and
        direction 'dx' as (3n, 1) arrays, 'alphas', 'iters' = index of the last iteration) plus
        'residuals' (||g|| / ||g(x_tilde)|| at the start of each iteration), 'pcg_iters' per
        iteration and the step's 'status' (0, or the skg_status of a failed solve or search)."""
        mass = _vertex_masses(M, self.X.shape[0])
        if mass is None:
            return None
        solver = self.stepper(h, mass, integrator)
        solver.params.tol = float(tolerance)
        solver.params.max_newton = int(max_iter)
        solver.params.do_line_search = int(do_line_search)
        solver.params.stop_rule = 1
        rec = None
        if return_info:
            cap = max(int(max_iter), 1)
            n3 = self.X.size
            rec = {"g": torch.empty((cap, n3), dtype=torch.float64, device=solver.mesh.device),
                   "dx": torch.empty((cap, n3), dtype=torch.float64, device=solver.mesh.device),
                   "alpha": np.zeros(cap), "res": np.zeros(cap), "pcg": np.zeros(cap, np.int32)}
            host = lambda a: a.ctypes.data_as(ctypes.c_void_p)
            rec["c"] = _lib.NewtonRecordC(capacity=cap, g=rec["g"].data_ptr(), dx=rec["dx"].data_ptr(),
                                          alpha_h=host(rec["alpha"]), residual_h=host(rec["res"]),
                                          pcg_iters_h=host(rec["pcg"]))
            solver.params.record = ctypes.pointer(rec["c"])
        try:
            if integrator == "bdf2":
                x_next, st = solver.step_host(xs[0], xs[1], x_prev2=xs[2], x_prev3=xs[3])
            else:
                x_next, st = solver.step_host(xs[0], xs[1])
        finally:
            solver.params.record = None
        if rec is None:
            return x_next
        k = int(st.newton_iters)
        g = rec["g"][:k].cpu().numpy()
        dx = rec["dx"][:k].cpu().numpy()
        info = {"g": [g[i].reshape(-1, 1) for i in range(k)], "dx": [dx[i].reshape(-1, 1) for i in range(k)],
                "alphas": [float(a) for a in rec["alpha"][:k]], "iters": k - 1,
                "residuals": [float(r) for r in rec["res"][:k]], "pcg_iters": [int(c) for c in rec["pcg"][:k]],
                "status": int(st.status)}
        return x_next, info


def _potential_of(*funcs):
    """The ElasticPotential whose energy, gradient and hessian methods these are, else None."""
    owners = [getattr(f, "__self__", None) for f in funcs]
    names = [getattr(getattr(f, "__func__", None), "__name__", None) for f in funcs]
    if (isinstance(owners[0], ElasticPotential) and all(o is owners[0] for o in owners)
            and names == ["energy", "gradient", "hessian"]):
        return owners[0]
    return None


def _vertex_masses(M, n: int):
    """Per-vertex masses of a diagonal (3n, 3n) mass matrix with equal entries per vertex, else None."""
    if sps.issparse(M):
        if M.shape != (3 * n, 3 * n):
            return None
        d = np.asarray(M.diagonal(), dtype=np.float64)
        if (sps.csr_matrix(M) - sps.diags(d)).tocsr().count_nonzero():
            return None
    else:
        A = np.asarray(M, dtype=np.float64)
        if A.shape != (3 * n, 3 * n):
            return None
        d = np.diagonal(A).copy()
        if np.count_nonzero(A - np.diag(d)):
            return None
    dv = d.reshape(n, 3)
    if not np.all(dv == dv[:, :1]):
        return None
    return dv[:, 0].copy()


def backward_euler(x_curr, x_prev, energy_func, gradient_func, hessian_func, M, h, tolerance: float = 1e-6,
                   max_iter: int = 1, do_line_search: bool = True, return_info: bool = False):
    """simkit ``backward_euler`` (integrators/backward_euler.py:27-91): minimise
    V(x) + 1/(2h^2) (x - x~)^T M (x - x~), x~ = 2 x_curr - x_prev, by ``newton_solver``.

    With the closures of an ``ElasticPotential`` and a lumped M (host arrays) the step runs on the
    device with the same Newton contract (``return_info`` gives simkit's info dict plus per-iteration
    residuals, PCG iterations and a status); otherwise the closures are called.
    """
    pot = _potential_of(energy_func, gradient_func, hessian_func)
    if pot is not None and all(isinstance(a, np.ndarray) for a in (x_curr, x_prev)):
        out = pot._device_step("be", M, h, tolerance, max_iter, do_line_search, (x_curr, x_prev), return_info)
        if out is not None:
            return out
    x_tilde = x_curr + h * ((x_curr - x_prev) / h)

    def energy(x):
        d = x - x_tilde
        return energy_func(x) + float((0.5 * (d.T @ (M @ d)) / h ** 2).item())

    def gradient(x):
        return gradient_func(x) + (M @ (x - x_tilde)) / h ** 2

    def hessian(x):
        return hessian_func(x) + M / h ** 2   # a device BlockMatrix stays on the device

    return newton_solver(x_tilde, energy, gradient, hessian, tolerance=tolerance, max_iter=max_iter,
                         do_line_search=do_line_search, return_info=return_info)


def bdf2(x_curr, x_prev, x_prev2, x_prev3, energy_func, gradient_func, hessian_func, M, h, tolerance: float = 1e-6,
         max_iter: int = 1, do_line_search: bool = True, return_info: bool = False):
    """simkit ``bdf2`` (integrators/bdf2.py:31-101): minimise V(x) + (9/4)/(2h^2) (x - x~)^T M (x - x~)
    with the BDF2 target x~ = (4/3) x_curr - (1/3) x_prev + (8h/9) v_curr - (2h/9) v_prev, velocities
    by the second-order backward difference (energies/kinetic.py:63-101), by ``newton_solver``.
    An ``ElasticPotential``'s closures with a lumped M take the device path, as in ``backward_euler``."""
    pot = _potential_of(energy_func, gradient_func, hessian_func)
    xs = (x_curr, x_prev, x_prev2, x_prev3)
    if pot is not None and all(isinstance(a, np.ndarray) for a in xs):
        out = pot._device_step("bdf2", M, h, tolerance, max_iter, do_line_search, xs, return_info)
        if out is not None:
            return out
    v_curr = (3.0 * x_curr - 4.0 * x_prev + x_prev2) / (2.0 * h)
    v_prev = (3.0 * x_prev - 4.0 * x_prev2 + x_prev3) / (2.0 * h)
    x_tilde = (4.0 / 3.0) * x_curr - (1.0 / 3.0) * x_prev + (8.0 * h / 9.0) * v_curr - (2.0 * h / 9.0) * v_prev
    c = 9.0 / 4.0

    def energy(x):
        d = x - x_tilde
        return energy_func(x) + float((0.5 * c * (d.T @ (M @ d)) / h ** 2).item())

    def gradient(x):
        return gradient_func(x) + c * (M @ (x - x_tilde)) / h ** 2

    def hessian(x):
        return hessian_func(x) + c * M / h ** 2   # a device BlockMatrix stays on the device

    return newton_solver(x_tilde, energy, gradient, hessian, tolerance=tolerance, max_iter=max_iter,
                         do_line_search=do_line_search, return_info=return_info)
