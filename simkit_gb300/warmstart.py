"""Learned warm start for batched backward-Euler Newton solves.

A 4-layer MLP (64 -> 256 -> 256 -> 256 -> 3, GELU, BF16 weights, FP32
accumulation) predicts, per vertex, what the second-order extrapolation
``u_tilde + corr_t`` (``corr_t`` = the previous step's Newton correction)
misses of the next Newton solution, in units of ``9.8 dt^2``, from per-vertex
state and a per-instance mean-pooled context (``skg_warmstart_features``).  Every GEMM of the forward
and backward passes runs on the tcgen05 tensor-core kernel
(``skg_mlp_gemm``); training uses Adam on FP32 master weights.

The network only proposes a starting point: ``BatchedBESolver.step`` keeps it
for an instance only if the gradient norm there is below the one at ``x_tilde``
(the residual-judged fallback) - otherwise that instance falls back to
``x_tilde`` - and Newton always runs to the same relative residual, measured
against ``||g(x_tilde)||``.  So the network changes the iteration
count, never the converged answer.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from ._lib import check

FEAT = 64
DIMS = [(64, 256), (256, 256), (256, 256), (256, 16)]   # (inputs, outputs); 3 of the last 16 are used
EPI_F32, EPI_BIAS_GELU, EPI_BF16 = 0, 1, 2


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _s():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _pad64(m):
    return (m + 63) // 64 * 64


class WarmStartMLP:
    """The network, its Adam state and its tensor-core forward / backward passes."""

    def __init__(self, seed=0, lr=1e-3, device="cuda"):
        self.lib = _lib.load()
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.W, self.b, self.W16, self.WT16 = [], [], [], []
        self.mW, self.vW, self.mb, self.vb = [], [], [], []
        for li, (k, n) in enumerate(DIMS):
            scale = math.sqrt(2.0 / k) * (0.1 if li == len(DIMS) - 1 else 1.0)
            w = (torch.randn(n, k, generator=g) * scale).to(device)
            if li == len(DIMS) - 1:
                w[3:] = 0.0                      # only 3 outputs are trained
            self.W.append(w.contiguous())
            self.b.append(torch.zeros(n, device=device))
            self.W16.append(w.bfloat16().contiguous())
            npad = max(n, 64)
            wt = torch.zeros(k, npad, dtype=torch.bfloat16, device=device)
            wt[:, :n] = w.T.bfloat16()
            self.WT16.append(wt)
            self.mW.append(torch.zeros_like(w))
            self.vW.append(torch.zeros_like(w))
            self.mb.append(torch.zeros(n, device=device))
            self.vb.append(torch.zeros(n, device=device))
        self.lr = lr
        self.t = 0
        self.err = torch.zeros(1, dtype=torch.int32, device=device)
        self.scratch = torch.zeros(2056, dtype=torch.float64, device=device)

    def refresh_bf16(self):
        """Rebuild the BF16 copies the GEMMs read (W and W^T, padded) from the FP32 masters - after
        the masters were loaded from a checkpoint (the Adam kernel keeps them in step otherwise)."""
        for li, (k, n) in enumerate(DIMS):
            self.W16[li].copy_(self.W[li].bfloat16())
            self.WT16[li].zero_()
            self.WT16[li][:, :n] = self.W[li].T.bfloat16()

    # -------------------------------------------------------------- GEMM
    def _gemm(self, A, B, Nc, epi, bias=None, out_f=None, out_z=None, out_h=None, Nstore=None, ld_out=None,
              splits=1):
        R, L = A.shape
        check(self.lib.skg_mlp_gemm(_p(A), R, A.stride(0), _p(B), Nc, B.stride(0), L, splits, epi, _p(bias),
                                    _p(out_f), _p(out_z), _p(out_h), Nc if Nstore is None else Nstore,
                                    Nc if ld_out is None else ld_out, _p(self.err), _s()))

    def forward(self, X, keep=False):
        """X: [M, 64] BF16 rows.  Returns Y [M, 16] FP32 (columns 0..2 are the prediction)."""
        M = X.shape[0]
        dev = X.device
        acts = [X]
        zs = []
        h = X
        for li in range(3):
            n = DIMS[li][1]
            z = torch.empty(M, n, dtype=torch.bfloat16, device=dev)
            hn = torch.empty(M, n, dtype=torch.bfloat16, device=dev)
            self._gemm(h, self.W16[li], n, EPI_BIAS_GELU, bias=self.b[li], out_z=z, out_h=hn)
            zs.append(z)
            acts.append(hn)
            h = hn
        y = torch.empty(1, M, 16, dtype=torch.float32, device=dev)
        self._gemm(h, self.W16[3], 16, EPI_F32, bias=self.b[3], out_f=y)
        if keep:
            self._cache = (acts, zs)
        return y[0]

    def _transpose_pad(self, A, Mp):
        """A [M, C] BF16 -> A^T [C, Mp] with zero columns beyond M."""
        M, C = A.shape
        out = torch.zeros(C, Mp, dtype=torch.bfloat16, device=A.device)
        check(self.lib.skg_mlp_transpose(_p(A), M, C, A.stride(0), _p(out), Mp, _s()))
        return out

    def _weight_grad(self, dZ, H, Mp):
        """dW [N, K] = dZ^T H, split over the rows of the batch (deterministic reduction)."""
        N = dZ.shape[1]
        K = H.shape[1]
        dZT = self._transpose_pad(dZ, Mp)
        HT = self._transpose_pad(H, Mp)
        kblocks = Mp // 64
        per = max(1, min(kblocks, (226 * 1024 - 1024) // (128 * 128 + K * 128)))
        splits = (kblocks + per - 1) // per
        Np = max(N, 16)
        if Np != N:        # A rows must exist for the tile: pad dZ^T rows
            pad = torch.zeros(Np, Mp, dtype=torch.bfloat16, device=dZ.device)
            pad[:N] = dZT
            dZT = pad
        part = torch.empty(splits, Np, K, dtype=torch.float32, device=dZ.device)
        self._gemm(dZT, HT, K, EPI_F32, out_f=part, splits=splits)
        dW = torch.empty(Np, K, dtype=torch.float32, device=dZ.device)
        check(self.lib.skg_mlp_reduce_splits(_p(part), splits, Np * K, _p(dW), _s()))
        return dW[:N]

    def backward(self, dY):
        """dY: [M, 64] BF16 loss gradient w.r.t. the outputs (columns >= 3 zero).  Returns (dW, db) lists."""
        acts, zs = self._cache
        M = dY.shape[0]
        Mp = _pad64(M)
        dWs, dbs = [None] * 4, [None] * 4
        # last (linear) layer
        dZ = dY[:, :16]
        dWs[3] = self._weight_grad(dZ.contiguous(), acts[3], Mp)
        db = torch.empty(16, dtype=torch.float32, device=dY.device)
        check(self.lib.skg_mlp_colsum(_p(dY), M, 16, dY.stride(0), _p(db), _s()))
        dbs[3] = db
        dH = torch.empty(M, 256, dtype=torch.bfloat16, device=dY.device)
        self._gemm(dY, self.WT16[3], 256, EPI_BF16, out_h=dH)
        for li in (2, 1, 0):
            n = DIMS[li][1]
            dZ = torch.empty(M, n, dtype=torch.bfloat16, device=dY.device)
            check(self.lib.skg_mlp_gelu_backward(_p(dH), _p(zs[li]), M * n, _p(dZ), _s()))
            dWs[li] = self._weight_grad(dZ, acts[li], Mp)
            db = torch.empty(n, dtype=torch.float32, device=dY.device)
            check(self.lib.skg_mlp_colsum(_p(dZ), M, n, n, _p(db), _s()))
            dbs[li] = db
            if li > 0:
                k = DIMS[li][0]
                dH = torch.empty(M, k, dtype=torch.bfloat16, device=dY.device)
                self._gemm(dZ, self.WT16[li], k, EPI_BF16, out_h=dH)
        return dWs, dbs

    def loss_and_grad(self, X, T):
        """MSE of the first 3 outputs against T [M, 3]; fills the cache; returns (loss, dY)."""
        Y = self.forward(X, keep=True)
        M = X.shape[0]
        dY = torch.zeros(M, 64, dtype=torch.bfloat16, device=X.device)
        loss = ctypes.c_double()
        check(self.lib.skg_mlp_mse(_p(Y), 16, _p(T), M, 3, _p(dY), 64, _p(self.scratch), ctypes.byref(loss), _s()))
        return loss.value, dY

    def adam_step(self, dWs, dbs):
        self.t += 1
        for li, (k, n) in enumerate(DIMS):
            npad = max(n, 64)
            if li == len(DIMS) - 1:
                dWs[li][3:] = 0.0
                dbs[li][3:] = 0.0
            check(self.lib.skg_mlp_adam(_p(self.W[li]), _p(dWs[li].contiguous()), _p(self.mW[li]), _p(self.vW[li]),
                                        n, k, self.lr, 0.9, 0.999, 1e-8, self.t, _p(self.W16[li]), k,
                                        _p(self.WT16[li]), npad, _s()))
            check(self.lib.skg_mlp_adam(_p(self.b[li]), _p(dbs[li].contiguous()), _p(self.mb[li]), _p(self.vb[li]),
                                        1, n, self.lr, 0.9, 0.999, 1e-8, self.t, None, 0, None, 0, _s()))

    def train_step(self, X, T):
        loss, dY = self.loss_and_grad(X, T)
        dWs, dbs = self.backward(dY)
        self.adam_step(dWs, dbs)
        return loss

    def predict(self, X):
        return self.forward(X, keep=False)


# ----------------------------------------------------------------- features
class FeatureBuilder:
    """Builds MLP input rows for every instance of a BatchedBESolver."""

    def __init__(self, solver, specs):
        self.s = solver
        m = solver.mesh
        dev = m.device
        self.lib = _lib.load()
        sc = []
        for sp in specs:
            E = float(np.mean(sp.ym)) if sp.ym is not None else 1e6
            nu = float(np.mean(sp.pr)) if sp.pr is not None else 0.45
            nx, ny, nz = sp.dims
            sc.append([math.log10(E) - 6.0, (nu - 0.4) * 10.0, nx / 16.0, ny / 16.0, nz / 48.0])
        self.inst_scalars = torch.tensor(sc, dtype=torch.float32, device=dev)
        self.vf = torch.empty(m.n, 16, dtype=torch.float32, device=dev)
        self.ctx = torch.empty(solver.n_inst, 32, dtype=torch.float32, device=dev)
        self.corr = torch.zeros(3 * m.n, dtype=torch.float64, device=dev)
        self.dt = solver.params.dt

    def features(self):
        s = self.s
        out = torch.empty(s.mesh.n, FEAT, dtype=torch.bfloat16, device=s.mesh.device)
        check(self.lib.skg_warmstart_features(_p(s.mesh.X), _p(s.u_curr), _p(s.u_prev), _p(self.corr),
                                              _p(s.f_ext), _p(s.mass), self.dt, s.mesh.n, _p(s.inst_rows),
                                              _p(s.vert_inst), s.n_inst, _p(self.inst_scalars), _p(self.vf),
                                              _p(self.ctx), _p(out), _s()))
        return out

    def u_tilde(self):
        return 2.0 * self.s.u_curr - self.s.u_prev

    def record_correction(self, ut):
        """after a step: corr = u_{t+1} - u_tilde_{t+1} (fed to the next step's features)"""
        self.corr.copy_(self.s.u_curr - ut)


def generate_frames(solver, specs, steps):
    """Run the plain batched solver ``steps`` steps; return per-step (features, targets, solver infos)."""
    fb = FeatureBuilder(solver, specs)
    lib = _lib.load()
    frames = []
    for _ in range(steps):
        X = fb.features()
        ut = fb.u_tilde()
        infos, total = solver.step()
        T = torch.empty(solver.mesh.n, 3, dtype=torch.float32, device=X.device)
        check(lib.skg_warmstart_targets(_p(solver.u_curr), _p(ut), _p(fb.corr), fb.dt, solver.mesh.n, _p(T), _s()))
        fb.record_correction(ut)
        frames.append((X, T, total))
    return frames, fb


def frame_rows(solver, frames, picks):
    """Concatenate the vertex rows of the (step, instance) frames in ``picks``."""
    rows = solver.inst_rows_host
    Xs, Ts = [], []
    for s, i in picks:
        X, T, _ = frames[s]
        Xs.append(X[rows[i]:rows[i + 1]])
        Ts.append(T[rows[i]:rows[i + 1]])
    return torch.cat(Xs).contiguous(), torch.cat(Ts).contiguous()


def train(mlp, solver, frames, epochs=2, batch_frames=64, seed=0, log=None):
    """Adam over random batches of ``batch_frames`` frames (each frame is one instance at one step)."""
    rng = np.random.default_rng(seed)
    all_frames = [(s, i) for s in range(len(frames)) for i in range(solver.n_inst)]
    losses = []
    for ep in range(epochs):
        order = rng.permutation(len(all_frames))
        for k in range(0, len(order) - batch_frames + 1, batch_frames):
            picks = [all_frames[j] for j in order[k:k + batch_frames]]
            X, T = frame_rows(solver, frames, picks)
            losses.append(mlp.train_step(X, T))
        if log:
            log(ep, losses[-1])
    return losses


def warm_step(solver, fb, mlp):
    """One batched step started from the network's prediction (with the residual-judged fallback).
    ``mlp=None`` starts from the plain second-order extrapolation u_tilde + corr."""
    lib = _lib.load()
    ut = fb.u_tilde()
    Y = mlp.predict(fb.features()) if mlp is not None else None
    uw = torch.empty_like(ut)
    check(lib.skg_warmstart_apply(_p(ut), _p(fb.corr), _p(Y), 16, _p(solver.pinned), fb.dt, solver.mesh.n, _p(uw),
                                  _s()))
    infos, total = solver.step(u_warm=uw)
    fb.record_correction(ut)
    return infos, total
