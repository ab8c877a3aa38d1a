"""Device-resident tet mesh: rest-shape operator, material and sparsity maps.

One ``TetMesh`` replaces what simkit precomputes per mesh for this path:
``deformation_jacobian`` (``simkit/deformation_jacobian.py:9-87``) becomes a
per-tet inverse rest edge matrix, ``volume`` (``simkit/volume.py:14-41``) a
per-tet signed volume (both computed by the ``skg_tet_setup`` kernel), and
the sparsity of ``J^T blockdiag(He) J`` (``snh.py:536-537``) a block pattern
with deterministic gather maps (``skg_pattern_build``).
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import TetMeshC, check


def _stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


# code of the per-tet block (a, b) in the assembly gather maps: 0..3 diagonal (a, a),
# 4..9 off-diagonal a < b, 10..15 the transpose of (b, a) for a > b
def _block_codes():
    off = lambda a, b: (b - 1) if a == 0 else ((b + 1) if a == 1 else 5)
    return [a if a == b else (4 + off(a, b) if a < b else 10 + off(b, a)) for a in range(4) for b in range(4)]


def device_pattern(tets: torch.Tensor, n: int):
    """Block pattern and gather maps of a tet mesh built with sorts on the tets' device.

    Same output as ``skg_pattern_build`` (block rows = vertices, columns sorted
    ascending; per slot the per-tet blocks in tet order; vertex -> tet*4+corner
    in tet order) for meshes without isolated vertices: one stable sort of the
    16 t (row, column) keys and one of the 4 t vertex keys.  Returns
    (rowptr, col, diag, row, hc_ptr, hc_src, v2t_ptr, v2t) as int32 tensors.
    """
    dev = tets.device
    t = tets.shape[0]
    a = tets.reshape(t, 4).long()
    vcount = torch.bincount(a.reshape(-1), minlength=n)
    if vcount.numel() != n or bool((vcount == 0).any()):
        raise ValueError("device pattern: every vertex must belong to a tet")
    rows = a[:, :, None].expand(t, 4, 4).reshape(-1)
    cols = a[:, None, :].expand(t, 4, 4).reshape(-1)
    codes = torch.tensor(_block_codes(), dtype=torch.long, device=dev)
    src = (16 * torch.arange(t, device=dev)[:, None] + codes[None, :]).reshape(-1)
    skey, perm = torch.sort(rows * n + cols, stable=True)
    hc_src = src[perm].int()
    new = torch.ones_like(skey, dtype=torch.bool)
    new[1:] = skey[1:] != skey[:-1]
    starts = torch.nonzero(new).reshape(-1)
    ukey = skey[starts]
    row = (ukey // n)
    col = (ukey % n)
    nb = int(starts.numel())
    hc_ptr = torch.cat([starts, torch.tensor([16 * t], device=dev)]).int()
    rowptr = torch.zeros(n + 1, dtype=torch.long, device=dev)
    rowptr[1:] = torch.cumsum(torch.bincount(row, minlength=n), 0)
    slots = torch.arange(nb, device=dev)
    diag = torch.empty(n, dtype=torch.long, device=dev)
    on = row == col
    diag[row[on]] = slots[on]
    vkey, vperm = torch.sort(a.reshape(-1), stable=True)
    v2t = vperm.int()
    v2t_ptr = torch.zeros(n + 1, dtype=torch.long, device=dev)
    v2t_ptr[1:] = torch.cumsum(vcount, 0)
    return (rowptr.int(), col.int(), diag.int(), row.int(), hc_ptr, hc_src, v2t_ptr.int(), v2t)


AUTO_COARSE = 3072   # coarse unknowns of box=None: a dense inverse of at most 38 MB


def coarse_aggregates(X, free_dof, rowptr, col, box=8, spacing=None, max_coarse=4096):
    """Aggregates and coarse-operator pattern of the two-level preconditioner.

    Vertices are grouped by the box of ``box`` x ``box`` x ``box`` mesh spacings their rest
    position falls in (``spacing`` defaults to (bounding-box volume / n)^(1/3), the cell size of a
    structured grid); each aggregate carries 3 translations and 3 rotations about its centroid.
    The box grows until the 6 unknowns per aggregate fit in ``max_coarse``.  ``box=None`` picks the
    finest box from 6 spacings up whose coarse space fits ``AUTO_COARSE`` unknowns (smaller boxes cut
    PCG iterations - on the 786,432-tet beam 42.3 per Newton solve with box 8, 37.6 with box 7 - while
    the dense coarse inverse grows with the square of the count).

    Returns a dict of host arrays: ``n_agg``; ``mode`` (n, 4) float32 whose w lane holds the uint32
    bits aggregate | free-DOF mask << 29; ``cb_ptr``, ``cb_slot`` (fine block slots grouped by
    coarse block, row-major over aggregate pairs), ``cb_rc`` (aggregate row, column per coarse
    block); and ``box``, the box size used."""
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    n = X.shape[0]
    free = np.asarray(free_dof, dtype=bool).reshape(n, 3)
    lo = X.min(axis=0)
    ext = np.maximum(X.max(axis=0) - lo, 1e-300)
    if spacing is None:
        spacing = float(np.prod(ext) / max(n, 1)) ** (1.0 / 3.0)
        # flat or thin meshes: fall back to the largest extent per vertex
        if not spacing > 0.0:
            spacing = float(ext.max()) / max(n, 1)
    if box is None:
        box, max_coarse = 6, min(max_coarse, AUTO_COARSE)
    while True:
        h = box * spacing
        ijk = np.floor((X - lo) / h + 0.5 / box).astype(np.int64)
        keys = (ijk[:, 0] * (ijk[:, 1].max() + 1) + ijk[:, 1]) * (ijk[:, 2].max() + 1) + ijk[:, 2]
        uk, agg = np.unique(keys, return_inverse=True)
        n_agg = uk.size
        if 6 * n_agg <= max_coarse:
            break
        box = box + 1 if max_coarse == AUTO_COARSE and box < 16 else box * 2
    agg = agg.astype(np.int64).reshape(-1)
    cnt = np.bincount(agg, minlength=n_agg).astype(np.float64)
    cen = np.stack([np.bincount(agg, weights=X[:, k], minlength=n_agg) for k in range(3)], 1) / cnt[:, None]
    d = X - cen[agg]
    rms = np.sqrt(np.bincount(agg, weights=(d * d).sum(1), minlength=n_agg) / cnt)
    rms = np.where(rms > 0.0, rms, 1.0)
    # fp16-exact offsets: the block records carry them packed as fp16 for the gathers
    d = (d / rms[agg][:, None]).astype(np.float16).astype(np.float32)
    mask = (free[:, 0].astype(np.uint32) | (free[:, 1].astype(np.uint32) << 1)
            | (free[:, 2].astype(np.uint32) << 2))
    bits = agg.astype(np.uint32) | (mask << np.uint32(29))
    mode = np.empty((n, 4), np.float32)
    mode[:, :3] = d
    mode[:, 3] = bits.view(np.float32)
    cb_ptr, cb_slot, cb_rc = _coarse_pattern(agg, n_agg, rowptr, col, n)
    return {"n_agg": int(n_agg), "mode": mode, "cb_ptr": cb_ptr, "cb_slot": cb_slot, "cb_rc": cb_rc, "box": box}


def _coarse_pattern(agg, n_agg, rowptr, col, n):
    rowptr = np.asarray(rowptr, dtype=np.int64)
    col = np.asarray(col, dtype=np.int64)
    row = np.repeat(np.arange(n, dtype=np.int64), np.diff(rowptr))
    ckey = agg[row] * n_agg + agg[col]
    order = np.argsort(ckey, kind="stable")
    ks = ckey[order]
    starts = np.flatnonzero(np.r_[True, ks[1:] != ks[:-1]])
    cb_keys = ks[starts]
    cb_ptr = np.r_[starts, ks.size].astype(np.int32)
    cb_rc = np.stack([cb_keys // n_agg, cb_keys % n_agg], 1).astype(np.int32).reshape(-1)
    return cb_ptr, order.astype(np.int32), cb_rc


def coarse_aggregates_inst(X, free_dof, rowptr, col, inst_rows, box=4, max_agg=127, spacing=None):
    """Per-instance aggregates of the two-level preconditioner for the thread-block-cluster PCG
    (one mesh is one instance; a batch has one per mesh).

    Each instance's vertices are grouped by boxes of ``box`` mesh spacings (grown until the instance
    has at most ``max_agg`` aggregates, so a local aggregate index fits 7 bits).  Offsets from the
    aggregate centroid are divided by the aggregate's largest |component| and quantised to k/64,
    k in [-64, 63]; those exact values are what every user of P sees.  Returns host arrays:
    ``n_agg``; ``mode`` (n, 4) float32 (offset, uint32 bits global aggregate | free mask << 29);
    ``colpack`` (n) uint32 = (k_x+64) | (k_y+64) << 7 | (k_z+64) << 14 | local aggregate << 21 |
    free mask << 28, the word the block records carry for their column; the coarse block
    pattern ``cb_ptr``, ``cb_slot``, ``cb_rc``; per instance ``inst_agg`` (n_inst + 1),
    ``agg_inst`` (n_agg), ``inst_moff`` (n_inst + 1, offsets of the padded dense blocks in
    floats), ``m_floats``, ``max_np``, ``boxes``."""
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    n = X.shape[0]
    free = np.asarray(free_dof, dtype=bool).reshape(n, 3)
    inst_rows = np.asarray(inst_rows, dtype=np.int64)
    ni = inst_rows.size - 1
    agg = np.empty(n, np.int64)
    local = np.empty(n, np.int64)
    d = np.empty((n, 3), np.float64)
    inst_agg = [0]
    boxes = []
    for i in range(ni):
        a, b = int(inst_rows[i]), int(inst_rows[i + 1])
        Xi = X[a:b]
        lo = Xi.min(axis=0)
        ext = np.maximum(Xi.max(axis=0) - lo, 1e-300)
        sp = spacing if spacing is not None else float(np.prod(ext) / max(b - a, 1)) ** (1.0 / 3.0)
        bx = box
        while True:
            h = bx * sp
            ijk = np.floor((Xi - lo) / h + 0.5 / bx).astype(np.int64)
            keys = (ijk[:, 0] * (ijk[:, 1].max() + 1) + ijk[:, 1]) * (ijk[:, 2].max() + 1) + ijk[:, 2]
            uk, la = np.unique(keys, return_inverse=True)
            if uk.size <= max_agg:
                break
            bx *= 2
        la = la.reshape(-1)
        na = uk.size
        cnt = np.bincount(la, minlength=na).astype(np.float64)
        cen = np.stack([np.bincount(la, weights=Xi[:, k], minlength=na) for k in range(3)], 1) / cnt[:, None]
        di = Xi - cen[la]
        mx = np.zeros(na)
        np.maximum.at(mx, la, np.abs(di).max(axis=1))
        di = di / np.where(mx > 0.0, mx, 1.0)[la][:, None]
        agg[a:b] = inst_agg[-1] + la
        local[a:b] = la
        d[a:b] = di
        inst_agg.append(inst_agg[-1] + na)
        boxes.append(bx)
    n_agg = inst_agg[-1]
    q = np.clip(np.rint(d * 64.0), -64, 63).astype(np.int64)
    mask = (free[:, 0].astype(np.uint32) | (free[:, 1].astype(np.uint32) << 1)
            | (free[:, 2].astype(np.uint32) << 2))
    mode = np.empty((n, 4), np.float32)
    mode[:, :3] = q / 64.0
    mode[:, 3] = (agg.astype(np.uint32) | (mask << np.uint32(29))).view(np.float32)
    colpack = ((q[:, 0] + 64) | ((q[:, 1] + 64) << 7) | ((q[:, 2] + 64) << 14) | (local << 21)
               | (mask.astype(np.int64) << 28)).astype(np.uint32)
    cb_ptr, cb_slot, cb_rc = _coarse_pattern(agg, n_agg, rowptr, col, n)
    inst_agg = np.asarray(inst_agg, np.int64)
    nps = ((6 * np.diff(inst_agg) + 31) // 32) * 32
    inst_moff = np.r_[0, np.cumsum(nps * nps)].astype(np.int64)
    agg_inst = np.repeat(np.arange(ni, dtype=np.int32), np.diff(inst_agg))
    return {"n_agg": int(n_agg), "mode": mode, "colpack": colpack, "cb_ptr": cb_ptr, "cb_slot": cb_slot,
            "cb_rc": cb_rc, "inst_agg": inst_agg.astype(np.int32), "agg_inst": agg_inst, "inst_moff": inst_moff,
            "m_floats": int(inst_moff[-1]), "max_np": int(nps.max()), "boxes": np.asarray(boxes)}


class TetMesh:
    """Rest mesh of n vertices and t tets on one GPU.

    Parameters
    ----------
    X : (n, 3) rest positions;  T : (t, 4) tets;  mu, lam : (t,) or (t, 1).
    """

    @classmethod
    def from_device(cls, X, tets, dinv, vol, mu, lam, pattern):
        """A mesh from device tensors: X (3n) f64, tets (t, 4) i32, dinv (9t) f64, vol (t) f64,
        mu, lam (t) f64 and ``pattern`` = (rowptr, col, diag, row, hc_ptr, hc_src, v2t_ptr, v2t)
        as produced by ``device_pattern`` (or the same maps concatenated with offsets)."""
        self = cls.__new__(cls)
        self.device = X.device
        self.n = X.numel() // 3
        self.t = tets.shape[0]
        self.X_host = None
        self.T_host = None
        self.X, self.tets, self.dinv, self.vol = X, tets, dinv, vol
        self.mu, self.lam = mu.contiguous(), lam.contiguous()
        self.dinv32 = dinv.float()
        self.mat32 = torch.stack([vol, self.mu, self.lam]).float().contiguous()
        (self.rowptr, self.col, self.diag, self.row, self.hc_ptr, self.hc_src, self.v2t_ptr, self.v2t) = pattern
        self.nb = int(self.col.numel())
        self.rowptr_host = None
        self.col_host = None
        self._set_c()
        self._scalar_perm = None
        return self

    def _set_upper(self):
        """Upper-triangle slot lists for the symmetric assembly (device, from the pattern): the slots
        (v, w) with w >= v, the slot of each one's transpose, and their contribution lists."""
        row, col = self.row.long(), self.col.long()
        up = col >= row
        slot = torch.nonzero(up).reshape(-1)
        keys = row * self.n + col                      # ascending: rows in order, columns sorted
        mirror = torch.searchsorted(keys, col[slot] * self.n + row[slot])
        hp = self.hc_ptr.long()
        cnt = (hp[1:] - hp[:-1])[slot]
        ptr = torch.zeros(slot.numel() + 1, dtype=torch.int64, device=row.device)
        ptr[1:] = torch.cumsum(cnt, 0)
        total = int(ptr[-1])
        idx = torch.repeat_interleave(hp[:-1][slot] - ptr[:-1], cnt, output_size=total)
        idx += torch.arange(total, device=row.device)
        self.up_slot, self.up_mirror = slot.int(), mirror.int()
        self.hcu_ptr, self.hcu_src = ptr.int(), self.hc_src[idx].contiguous()

    def _set_c(self):
        if not hasattr(self, "material"):
            self.material = 0
        if getattr(self, "up_slot", None) is None:
            self._set_upper()
        self.c = TetMeshC(
            n_verts=self.n, n_tets=self.t, n_blocks=self.nb,
            tets=self.tets.data_ptr(), dinv=self.dinv.data_ptr(), dinv32=self.dinv32.data_ptr(),
            vol=self.vol.data_ptr(), mu=self.mu.data_ptr(), lam=self.lam.data_ptr(), mat32=self.mat32.data_ptr(),
            bsr_rowptr=self.rowptr.data_ptr(), bsr_col=self.col.data_ptr(), bsr_diag=self.diag.data_ptr(),
            bsr_row=self.row.data_ptr(), hc_ptr=self.hc_ptr.data_ptr(), hc_src=self.hc_src.data_ptr(),
            v2t_ptr=self.v2t_ptr.data_ptr(), v2t=self.v2t.data_ptr(), material=self.material,
            n_upper=self.up_slot.numel(), up_slot=self.up_slot.data_ptr(), up_mirror=self.up_mirror.data_ptr(),
            hcu_ptr=self.hcu_ptr.data_ptr(), hcu_src=self.hcu_src.data_ptr())

    def __init__(self, X, T, mu, lam, device="cuda"):
        lib = _lib.load()
        X = np.ascontiguousarray(np.asarray(X, dtype=np.float64).reshape(-1, 3))
        T = np.ascontiguousarray(np.asarray(T).reshape(-1, 4).astype(np.int32))
        self.n = n = X.shape[0]
        self.t = t = T.shape[0]
        if t == 0:
            raise ValueError("mesh has no tets")
        if T.min() < 0 or T.max() >= n:
            raise ValueError("tet indices out of range")
        self.device = torch.device(device)
        dev = self.device
        self.X_host = X
        self.T_host = T
        self.X = torch.from_numpy(X.reshape(-1)).to(dev)
        self.tets = torch.from_numpy(T).to(dev)
        self.dinv = torch.empty(9 * t, dtype=torch.float64, device=dev)
        self.vol = torch.empty(t, dtype=torch.float64, device=dev)
        check(lib.skg_tet_setup(_ptr(self.X), _ptr(self.tets), n, t, _ptr(self.dinv), _ptr(self.vol), _stream_ptr()))
        # simkit's deformation_jacobian raises on a singular rest edge matrix (np.linalg.inv); the
        # device setup leaves a zero or non-finite volume and shape operator there instead
        bad = (self.vol == 0) | ~torch.isfinite(self.vol) | ~torch.isfinite(self.dinv.view(9, t)).all(dim=0)
        if bool(bad.any()):
            e = int(torch.nonzero(bad)[0, 0])
            raise ValueError(f"tet {e} is degenerate at rest (signed volume {float(self.vol[e]):.3e})")
        self.mu = torch.as_tensor(np.asarray(mu, dtype=np.float64).reshape(-1), device=dev).contiguous()
        self.lam = torch.as_tensor(np.asarray(lam, dtype=np.float64).reshape(-1), device=dev).contiguous()
        if self.mu.numel() != t or self.lam.numel() != t:
            raise ValueError("mu and lam need one value per tet")
        self.dinv32 = self.dinv.float()
        self.mat32 = torch.stack([self.vol, self.mu, self.lam]).float().contiguous()
        # pattern on the host (integer work, once per mesh)
        nb = ctypes.c_int64(0)
        Tp = T.ctypes.data_as(ctypes.c_void_p)
        check(lib.skg_pattern_build(Tp, n, t, ctypes.byref(nb), None, None, None, None, None, None, None))
        nb = nb.value
        self.nb = nb
        rowptr = np.empty(n + 1, np.int32)
        col = np.empty(nb, np.int32)
        diag = np.empty(n, np.int32)
        hc_ptr = np.empty(nb + 1, np.int32)
        hc_src = np.empty(16 * t, np.int32)
        v2t_ptr = np.empty(n + 1, np.int32)
        v2t = np.empty(4 * t, np.int32)
        a = lambda x: x.ctypes.data_as(ctypes.c_void_p)
        check(lib.skg_pattern_build(Tp, n, t, ctypes.byref(ctypes.c_int64(0)), a(rowptr), a(col), a(diag),
                                    a(hc_ptr), a(hc_src), a(v2t_ptr), a(v2t)))
        self.rowptr_host = rowptr
        self.col_host = col
        row = np.repeat(np.arange(n, dtype=np.int32), np.diff(rowptr))
        up = lambda x: torch.from_numpy(x).to(dev)
        self.rowptr, self.col, self.diag, self.row = up(rowptr), up(col), up(diag), up(row)
        self.hc_ptr, self.hc_src, self.v2t_ptr, self.v2t = up(hc_ptr), up(hc_src), up(v2t_ptr), up(v2t)
        self._set_c()
        self._scalar_perm = None

    def check_orientation(self):
        """Raise ValueError if a tet is inverted at rest (negative signed volume): its energy would
        enter the potential with a negative weight and Newton would maximise it."""
        neg = self.vol < 0
        if bool(neg.any()):
            e = int(torch.nonzero(neg)[0, 0])
            raise ValueError(f"tet {e} is inverted at rest (signed volume {float(self.vol[e]):.3e}); "
                             "swap two of its vertices")

    # ----------------------------------------------------------------- utils
    def set_coarse(self, free_dof, box=8, spacing=None):
        """Attach two-level preconditioner data (aggregates of ``box``^3 mesh spacings, 6 rigid
        modes each) built from the rest positions, the free-DOF mask (3n, True = free) and the
        block pattern.  Workspaces sized before this call are too small afterwards."""
        if self.X_host is None:
            self.X_host = self.X.cpu().numpy().reshape(-1, 3)
        if self.rowptr_host is None:
            self.rowptr_host = self.rowptr.cpu().numpy()
            self.col_host = self.col.cpu().numpy()
        cd = coarse_aggregates(self.X_host, free_dof, self.rowptr_host, self.col_host, box=box, spacing=spacing)
        up = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(self.device)
        self.coarse = {k: (up(v) if isinstance(v, np.ndarray) else v) for k, v in cd.items()}
        self._coarse_c = _lib.CoarseC(
            n_agg=cd["n_agg"], n_cblocks=int(cd["cb_ptr"].size - 1), mode=self.coarse["mode"].data_ptr(),
            cb_ptr=self.coarse["cb_ptr"].data_ptr(), cb_slot=self.coarse["cb_slot"].data_ptr(),
            cb_rc=self.coarse["cb_rc"].data_ptr())
        self.c.coarse = ctypes.pointer(self._coarse_c)
        return cd["n_agg"], cd["box"]

    def set_coarse_inst(self, free_dof, inst_rows=None, box=4):
        """Attach per-instance two-level data for the cluster PCG (``inst_rows``: instance vertex
        offsets, default one instance).  Workspaces sized before this call are too small afterwards."""
        if self.X_host is None:
            self.X_host = self.X.cpu().numpy().reshape(-1, 3)
        if self.rowptr_host is None:
            self.rowptr_host = self.rowptr.cpu().numpy()
            self.col_host = self.col.cpu().numpy()
        if inst_rows is None:
            inst_rows = np.array([0, self.n])
        cd = coarse_aggregates_inst(self.X_host, free_dof, self.rowptr_host, self.col_host, inst_rows, box=box)
        up = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(self.device)
        self.coarse = {k: (up(v) if isinstance(v, np.ndarray) and k != "boxes" else v) for k, v in cd.items()}
        ptr = lambda k: self.coarse[k].data_ptr()
        self._coarse_c = _lib.CoarseC(
            n_agg=cd["n_agg"], n_cblocks=int(cd["cb_ptr"].size - 1), mode=ptr("mode"), cb_ptr=ptr("cb_ptr"),
            cb_slot=ptr("cb_slot"), cb_rc=ptr("cb_rc"), n_inst=int(cd["inst_agg"].size - 1), max_np=cd["max_np"],
            m_floats=cd["m_floats"], inst_agg=ptr("inst_agg"), agg_inst=ptr("agg_inst"), inst_moff=ptr("inst_moff"),
            colpack=ptr("colpack"))
        self.c.coarse = ctypes.pointer(self._coarse_c)
        return cd["n_agg"], cd["boxes"]

    def set_coarse_device(self, t):
        """Attach per-instance two-level data already on the device: ``t`` holds ``mode`` (n, 4)
        float32, ``colpack`` (n) int32/uint32, ``cb_ptr``, ``cb_slot``, ``cb_rc``, ``inst_agg``,
        ``agg_inst`` (int32) and ``inst_moff`` (int64), as ``coarse_aggregates_inst`` lays them out."""
        ia = t["inst_agg"].cpu().numpy()
        nps = ((6 * np.diff(ia) + 31) // 32) * 32
        self.coarse = dict(t)
        ptr = lambda k: self.coarse[k].data_ptr()
        self._coarse_c = _lib.CoarseC(
            n_agg=int(ia[-1]), n_cblocks=int(t["cb_ptr"].numel() - 1), mode=ptr("mode"), cb_ptr=ptr("cb_ptr"),
            cb_slot=ptr("cb_slot"), cb_rc=ptr("cb_rc"), n_inst=int(ia.size - 1), max_np=int(nps.max()),
            m_floats=int((nps.astype(np.int64) ** 2).sum()), inst_agg=ptr("inst_agg"), agg_inst=ptr("agg_inst"),
            inst_moff=ptr("inst_moff"), colpack=ptr("colpack"))
        self.c.coarse = ctypes.pointer(self._coarse_c)

    def clear_coarse(self):
        self.c.coarse = None
        self.coarse = None
        self._coarse_c = None

    def set_energy(self, material):
        """Elastic energy of every tet: 0 / 'stable-neo-hookean', 1 / 'macklin-mueller-neo-hookean',
        2 / 'arap', 3 / 'fcr', 4 / 'linear-elasticity'."""
        code = {"stable-neo-hookean": 0, "macklin-mueller-neo-hookean": 1, "arap": 2, "fcr": 3,
                "linear-elasticity": 4}.get(material, material)
        if code not in (0, 1, 2, 3, 4):
            raise ValueError(f"unknown material {material!r}")
        self.material = code
        self.c.material = code

    def set_material(self, mu, lam, vol=None):
        """Replace per-tet mu, lam (and quadrature weights vol) in place."""
        def dev(a):
            a = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.asarray(a, dtype=np.float64))
            a = a.to(device=self.device, dtype=torch.float64).reshape(-1)
            if a.numel() != self.t:
                raise ValueError("material arrays need one value per tet")
            return a
        self.mu.copy_(dev(mu))
        self.lam.copy_(dev(lam))
        if vol is not None:
            self.vol.copy_(dev(vol))
        self.mat32.copy_(torch.stack([self.vol, self.mu, self.lam]).float())

    def workspace(self, precision) -> torch.Tensor:
        nbytes = _lib.load().skg_assembly_workspace_size(ctypes.byref(self.c), precision)
        if nbytes < 0:
            raise ValueError(_lib.last_error())
        return torch.empty(int(nbytes), dtype=torch.uint8, device=self.device)

    def scalar_pattern(self):
        """(indptr, indices, perm): scalar CSR pattern of the block matrix and the
        permutation taking block values (entry-major layout) to CSR data order."""
        if self._scalar_perm is None:
            if self.rowptr_host is None:
                self.rowptr_host = self.rowptr.cpu().numpy()
                self.col_host = self.col.cpu().numpy()
            rp = self.rowptr_host.astype(np.int64)
            col = self.col_host.astype(np.int64)
            n = self.n
            K = np.diff(rp)
            # scalar row 3v+i holds, for blocks k (sorted columns) and j, value
            # val[9 rp_v + (3i+j) K_v + k]
            vrow = np.repeat(np.arange(n), K)          # block row of each slot
            kloc = np.arange(col.size) - rp[vrow]     # local index in its row
            indptr = np.zeros(3 * n + 1, np.int64)
            indptr[1:] = np.repeat(3 * K, 3).cumsum()
            indices = np.empty(9 * col.size, np.int64)
            perm = np.empty(9 * col.size, np.int64)
            for i in range(3):
                # position of (slot, i, j) in CSR: indptr[3v+i] + 3 kloc + j
                base = indptr[3 * vrow + i] + 3 * kloc
                for j in range(3):
                    indices[base + j] = 3 * col + j
                    perm[base + j] = 9 * rp[vrow] + (3 * i + j) * K[vrow] + kloc
            self._scalar_perm = (indptr, indices, perm)
        return self._scalar_perm

    def diag_value_index(self) -> torch.Tensor:
        """(3n,) device positions, in the entry-major block values, of the scalar diagonal entries
        (3v + i, 3v + i)."""
        if getattr(self, "_diag_idx", None) is None:
            rp = self.rowptr.long()
            K = rp[1:] - rp[:-1]
            base = 9 * rp[:-1] + (self.diag.long() - rp[:-1])
            self._diag_idx = torch.stack([base + 4 * i * K for i in range(3)], dim=1).reshape(-1).contiguous()
        return self._diag_idx

    def block_values_to_csr(self, val: torch.Tensor):
        """scipy CSR (3n x 3n) from device block values."""
        import scipy.sparse as sps
        indptr, indices, perm = self.scalar_pattern()
        data = val.double().cpu().numpy()[perm]
        return sps.csr_matrix((data, indices, indptr), shape=(3 * self.n, 3 * self.n))
