"""The library's tcgen05 tensor-core path: one 128 x N x K product with the
operands in the K-major core-matrix layout, accumulated in tensor memory and
read back (mk_tc_gemm), against float64 products of the same 16-bit
operands. The products of 16-bit values are exact in FP32; the FP32
accumulation over K <= 128 terms is the only rounding (relative 1e-6)."""
import numpy as np
import pytest
import torch

from mosaic_gb300 import _lib, engine

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [torch.float16, torch.bfloat16])
@pytest.mark.parametrize("N,K", [(16, 16), (32, 64), (64, 32), (128, 128), (256, 48), (48, 112)])
def test_tc_gemm_matches_float64(cuda, dtype, N, K):
    L = _lib.load()
    g = torch.Generator().manual_seed(N * 1000 + K)
    A = torch.randn(128, K, generator=g).to(dtype)
    B = torch.randn(N, K, generator=g).to(dtype)
    Ad, Bd = A.to(cuda).contiguous(), B.to(cuda).contiguous()
    C = torch.full((128, N), float("nan"), dtype=torch.float32, device=cuda)
    _lib.check(L.mk_tc_gemm(N, K, int(dtype == torch.bfloat16), Ad.data_ptr(), Bd.data_ptr(),
                            C.data_ptr(), engine._stream_handle()))
    engine.sync()
    ref = A.double() @ B.double().T
    got = C.cpu().double()
    assert torch.isfinite(got).all()
    assert float((got - ref).abs().max()) <= 1e-6 * float(ref.abs().max()) * K ** 0.5 + 1e-6


def test_tc_gemm_rejects_bad_shapes(cuda):
    L = _lib.load()
    buf = torch.zeros(128 * 256, dtype=torch.float16, device=cuda)
    out = torch.zeros(128 * 256, dtype=torch.float32, device=cuda)
    for N, K in ((8, 16), (24, 16), (512, 16), (16, 8), (16, 256)):
        assert L.mk_tc_gemm(N, K, 0, buf.data_ptr(), buf.data_ptr(), out.data_ptr(),
                            engine._stream_handle()) == _lib.MK_EINVAL, (N, K)
