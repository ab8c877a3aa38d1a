"""The warm-start MLP's tensor-core GEMM and helper kernels against plain torch
FP32 references of the same ops.

Tolerances: GEMM products of BF16 inputs are exact in FP32; only the
accumulation order differs, so FP32 outputs agree to 1e-5 relative (to the
output's scale); BF16 outputs to 1e-2 relative.
"""

import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


@pytest.fixture(scope="module")
def lib():
    from simkit_gb300 import _lib
    return _lib.load()


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _gemm(lib, A, B, Nc, epi=0, bias=None, splits=1, Nstore=None, ld_out=None):
    R, L = A.shape
    Nstore = Nc if Nstore is None else Nstore
    ld_out = Nstore if ld_out is None else ld_out
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    out_f = out_z = out_h = None
    if epi == 0:
        out_f = torch.full((splits, R, ld_out), float("nan"), dtype=torch.float32, device="cuda")
    else:
        out_h = torch.full((R, ld_out), float("nan"), dtype=torch.bfloat16, device="cuda")
        if epi == 1:
            out_z = torch.full((R, ld_out), float("nan"), dtype=torch.bfloat16, device="cuda")
    st = lib.skg_mlp_gemm(_p(A), R, A.stride(0), _p(B), Nc, B.stride(0), L, splits, epi, _p(bias), _p(out_f),
                          _p(out_z), _p(out_h), Nstore, ld_out, _p(err), _stream())
    from simkit_gb300 import _lib
    assert st == 0, _lib.last_error()
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return out_f, out_z, out_h


@pytest.mark.parametrize("R,L,Nc", [(128, 64, 16), (300, 64, 64), (1000, 256, 256), (777, 128, 48)])
def test_gemm_fp32_epilogue_matches_torch(lib, R, L, Nc):
    g = torch.Generator(device="cuda").manual_seed(R + L + Nc)
    A = torch.randn(R, L, generator=g, device="cuda").bfloat16()
    B = torch.randn(Nc, L, generator=g, device="cuda").bfloat16()
    bias = torch.randn(Nc, generator=g, device="cuda")
    out, _, _ = _gemm(lib, A, B, Nc, epi=0, bias=bias)
    ref = A.float() @ B.float().T + bias
    err = (out[0] - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-5, err


def test_gemm_split_k_and_reduction(lib):
    R, Nc, L, splits = 256, 64, 64 * 40, 10
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn(R, L, generator=g, device="cuda").bfloat16()
    B = torch.randn(Nc, L, generator=g, device="cuda").bfloat16()
    part, _, _ = _gemm(lib, A, B, Nc, epi=0, splits=splits)
    out = torch.empty(R, Nc, dtype=torch.float32, device="cuda")
    assert lib.skg_mlp_reduce_splits(_p(part), splits, R * Nc, _p(out), _stream()) == 0
    ref = A.float() @ B.float().T
    assert (out - ref).abs().max().item() / ref.abs().max().item() < 1e-5


def test_gemm_gelu_epilogue(lib):
    R, L, Nc = 500, 128, 256
    g = torch.Generator(device="cuda").manual_seed(6)
    A = (0.3 * torch.randn(R, L, generator=g, device="cuda")).bfloat16()
    B = (0.3 * torch.randn(Nc, L, generator=g, device="cuda")).bfloat16()
    bias = torch.randn(Nc, generator=g, device="cuda")
    _, z, h = _gemm(lib, A, B, Nc, epi=1, bias=bias)
    zr = A.float() @ B.float().T + bias
    hr = torch.nn.functional.gelu(zr, approximate="tanh")
    assert (z.float() - zr).abs().max().item() <= 1e-2 * zr.abs().max().item()
    assert (h.float() - hr).abs().max().item() <= 1e-2 * hr.abs().max().item()


def test_helpers_match_torch(lib):
    g = torch.Generator(device="cuda").manual_seed(7)
    X = torch.randn(333, 96, generator=g, device="cuda").bfloat16()
    XT = torch.empty(96, 333, dtype=torch.bfloat16, device="cuda")
    assert lib.skg_mlp_transpose(_p(X), 333, 96, 96, _p(XT), 333, _stream()) == 0
    torch.cuda.synchronize()
    assert torch.equal(XT, X.T.contiguous())
    db = torch.empty(96, dtype=torch.float32, device="cuda")
    assert lib.skg_mlp_colsum(_p(X), 333, 96, 96, _p(db), _stream()) == 0
    torch.cuda.synchronize()
    assert torch.allclose(db, X.float().sum(0), rtol=1e-4, atol=1e-3)
    Z = torch.randn(1000, generator=g, device="cuda").bfloat16()
    dH = torch.randn(1000, generator=g, device="cuda").bfloat16()
    dZ = torch.empty_like(Z)
    assert lib.skg_mlp_gelu_backward(_p(dH), _p(Z), 1000, _p(dZ), _stream()) == 0
    zz = Z.float().requires_grad_(True)
    torch.nn.functional.gelu(zz, approximate="tanh").backward(dH.float())
    torch.cuda.synchronize()
    assert (dZ.float() - zz.grad).abs().max().item() <= 1e-2 * zz.grad.abs().max().item()
