"""The tcgen05 GEMM (mk_gemm_tc) against float64 products of the same BF16
operands: every operand layout the surrogate uses (k-contiguous,
m/n-contiguous, strided), ragged sizes, the fused epilogue (bias, ReLU,
accumulate, ReLU mask, row scale, row map), split K, and agreement with the
mma.sync GEMM (mk_gemm_bf16). Products of BF16 values are exact in FP32;
the FP32 accumulation is the only rounding."""
import numpy as np
import pytest
import torch

from mosaic_gb300 import _lib, engine

pytestmark = pytest.mark.gpu

ACC, BIAS, RELU = 1, 2, 4


def _p(t):
    return t.data_ptr() if t is not None else None


def _gemm_tc(M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, bias=None, flags=0, Cb=None, ldcb=0,
             mask=None, ldm=0, row_scale=None, row_map=None):
    L = _lib.load()
    _lib.check(L.mk_gemm_tc(M, N, K, _p(A), sam, sak, _p(B), sbk, sbn, _p(C), ldc, _p(bias), flags,
                            _p(Cb), ldcb, _p(mask), ldm, _p(row_scale), _p(row_map),
                            engine._stream_handle()))
    engine.sync()
    _lib.check(L.mk_sync_status(engine._stream_handle()))


def _tol(ref, K):
    return 2e-6 * float(ref.abs().max()) * max(K, 1) ** 0.5 + 1e-6


def _operands(rng, M, N, K, cuda):
    A = torch.tensor(rng.standard_normal((M, K)), dtype=torch.float32).bfloat16()
    W = torch.tensor(rng.standard_normal((N, K)), dtype=torch.float32).bfloat16()
    return A, W, A.to(cuda), W.to(cuda)


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (37, 70, 45), (676, 256, 256), (300, 2100, 72),
                                   (130, 17, 300), (1, 8, 8)])
def test_forward_layout_bias_relu(cuda, M, N, K):
    """C = relu(A W^T + b) with A (M, K), W (N, K) both k-contiguous; the
    bf16 copy too."""
    rng = np.random.default_rng(M + N + K)
    A, W, Ad, Wd = _operands(rng, M, N, K, cuda)
    bias = torch.tensor(rng.standard_normal(N), dtype=torch.float32)
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device=cuda)
    Cb = torch.empty((M, N), dtype=torch.bfloat16, device=cuda)
    _gemm_tc(M, N, K, Ad, K, 1, Wd, 1, K, C, N, bias.to(cuda), BIAS | RELU, Cb, N)
    ref = torch.relu(A.double() @ W.double().T + bias.double())
    assert float((C.cpu().double() - ref).abs().max()) <= _tol(ref, K)
    assert torch.allclose(Cb.cpu().double(), ref, rtol=1e-2, atol=1e-2 * float(ref.abs().max()))


@pytest.mark.parametrize("M,N,K", [(37, 70, 45), (676, 256, 256), (200, 40, 130)])
def test_input_gradient_layout_accumulate_and_mask(cuda, M, N, K):
    """G (M, N) @ W (N, K) -> (M, K): B n-contiguous; accumulated onto a
    preset C, and with the ReLU mask of a layer's outputs."""
    rng = np.random.default_rng(2 * M + K)
    G = torch.tensor(rng.standard_normal((M, N)), dtype=torch.float32).bfloat16()
    W = torch.tensor(rng.standard_normal((N, K)), dtype=torch.float32).bfloat16()
    Gd, Wd = G.to(cuda), W.to(cuda)
    D = torch.full((M, K), 0.5, dtype=torch.float32, device=cuda)
    _gemm_tc(M, K, N, Gd, N, 1, Wd, K, 1, D, K, flags=ACC)
    ref = G.double() @ W.double() + 0.5
    assert float((D.cpu().double() - ref).abs().max()) <= _tol(ref, N)
    post = torch.tensor(rng.standard_normal((M, K)), dtype=torch.float32)
    E = torch.empty((M, K), dtype=torch.float32, device=cuda)
    Eb = torch.empty((M, K), dtype=torch.bfloat16, device=cuda)
    _gemm_tc(M, K, N, Gd, N, 1, Wd, K, 1, E, K, Cb=Eb, ldcb=K, mask=post.to(cuda), ldm=K)
    ref = (G.double() @ W.double()) * (post.double() > 0)
    assert float((E.cpu().double() - ref).abs().max()) <= _tol(ref, N)
    assert torch.equal(Eb.cpu(), E.cpu().bfloat16())


@pytest.mark.parametrize("M,N,K", [(256, 256, 676), (37, 70, 45), (64, 72, 1867), (256, 32, 600)])
def test_weight_gradient_layout_split_k(cuda, M, N, K):
    """G^T (M = outputs, K = batch) @ X (K, N): A m-contiguous, B
    n-contiguous, long K split over CTAs that add into C."""
    rng = np.random.default_rng(3 * M + K)
    G = torch.tensor(rng.standard_normal((K, M)), dtype=torch.float32).bfloat16()
    X = torch.tensor(rng.standard_normal((K, N)), dtype=torch.float32).bfloat16()
    E = torch.full((M, N), float("nan"), dtype=torch.float32, device=cuda)
    _gemm_tc(M, N, K, G.to(cuda), 1, M, X.to(cuda), N, 1, E, N)
    ref = G.double().T @ X.double()
    assert float((E.cpu().double() - ref).abs().max()) <= _tol(ref, K)


def test_strided_operands(cuda):
    """Operands with strides that allow no 16-byte loads (odd leading
    dimensions, a view into a wider array)."""
    rng = np.random.default_rng(7)
    M, N, K = 90, 33, 31
    A_full = torch.tensor(rng.standard_normal((M, K + 3)), dtype=torch.float32).bfloat16()
    B_full = torch.tensor(rng.standard_normal((K, N + 5)), dtype=torch.float32).bfloat16()
    C = torch.empty((M, N), dtype=torch.float32, device=cuda)
    _gemm_tc(M, N, K, A_full.to(cuda), K + 3, 1, B_full.to(cuda), N + 5, 1, C, N)
    ref = A_full[:, :K].double() @ B_full[:, :N].double()
    assert float((C.cpu().double() - ref).abs().max()) <= _tol(ref, K)


def test_row_scale_and_row_map(cuda):
    """The decode epilogue: relu(A B + bias) * scale[m] stored at row
    row_map[m] of a larger output; rows not mapped keep their contents."""
    rng = np.random.default_rng(9)
    M, N, K = 300, 2304, 96
    A = torch.tensor(rng.standard_normal((M, K)), dtype=torch.float32).bfloat16()
    Bt = torch.tensor(rng.standard_normal((N, K)), dtype=torch.float32).bfloat16()
    bias = torch.tensor(rng.standard_normal(N), dtype=torch.float32)
    scale = torch.tensor(rng.uniform(0.5, 2.0, M), dtype=torch.float32)
    rows = torch.tensor(rng.permutation(2 * M)[:M], dtype=torch.int64)
    out = torch.full((2 * M, N), -7.0, dtype=torch.float32, device=cuda)
    _gemm_tc(M, N, K, A.to(cuda), K, 1, Bt.to(cuda), 1, K, out, N, bias.to(cuda), BIAS | RELU,
             row_scale=scale.to(cuda), row_map=rows.to(cuda))
    ref = torch.relu(A.double() @ Bt.double().T + bias.double()) * scale.double()[:, None]
    got = out.cpu().double()
    assert float((got[rows] - ref).abs().max()) <= _tol(ref, K) * 2
    untouched = np.setdiff1d(np.arange(2 * M), rows.numpy())
    assert bool((got[untouched] == -7.0).all())


def test_matches_the_mma_sync_gemm(cuda):
    """Same operands through mk_gemm_bf16 (mma.sync) and mk_gemm_tc
    (tcgen05): equal to FP32 accumulation-order rounding."""
    L = _lib.load()
    rng = np.random.default_rng(11)
    M, N, K = 676, 256, 256
    A, W, Ad, Wd = _operands(rng, M, N, K, cuda)
    bias = torch.tensor(rng.standard_normal(N), dtype=torch.float32, device=cuda)
    C1 = torch.empty((M, N), dtype=torch.float32, device=cuda)
    C2 = torch.empty((M, N), dtype=torch.float32, device=cuda)
    _lib.check(L.mk_gemm_bf16(M, N, K, _p(Ad), K, 1, _p(Wd), 1, K, _p(C1), N, _p(bias), BIAS | RELU,
                              None, 0, engine._stream_handle()))
    _gemm_tc(M, N, K, Ad, K, 1, Wd, 1, K, C2, N, bias, BIAS | RELU)
    assert float((C1 - C2).abs().max()) <= 1e-5 * float(C1.abs().max())


def test_rejects_bad_arguments(cuda):
    L = _lib.load()
    buf = torch.zeros(64, dtype=torch.bfloat16, device=cuda)
    out = torch.zeros(64, dtype=torch.float32, device=cuda)
    rows = torch.zeros(8, dtype=torch.int64, device=cuda)
    sh = engine._stream_handle()
    assert L.mk_gemm_tc(0, 8, 8, _p(buf), 8, 1, _p(buf), 1, 8, _p(out), 8, None, 0, None, 0,
                        None, 0, None, None, sh) == _lib.MK_EINVAL
    assert L.mk_gemm_tc(8, 8, 8, _p(buf), 8, 1, _p(buf), 1, 8, None, 8, None, 0, None, 0,
                        None, 0, None, None, sh) == _lib.MK_EINVAL
    assert L.mk_gemm_tc(8, 8, 8, _p(buf), 8, 1, _p(buf), 1, 8, _p(out), 8, None, ACC, None, 0,
                        None, 0, None, _p(rows), sh) == _lib.MK_EINVAL


def test_groups_shared_input_and_split_k(cuda):
    """Three products in one launch (mk_gemm_tc_groups): a shared A (group
    stride 0) against per-group B, bias and output; and per-group long-K
    weight-gradient products split over CTAs."""
    import ctypes
    L = _lib.load()
    rng = np.random.default_rng(13)
    G, M, N, K = 3, 200, 96, 72
    A = torch.tensor(rng.standard_normal((M, K)), dtype=torch.float32).bfloat16()
    W = torch.tensor(rng.standard_normal((G, N, K)), dtype=torch.float32).bfloat16()
    bias = torch.tensor(rng.standard_normal((G, N)), dtype=torch.float32)
    C = torch.full((G, M, N), float("nan"), dtype=torch.float32, device=cuda)
    gs = (ctypes.c_longlong * 6)(0, N * K, M * N, 0, N, 0)
    Ad, Wd, bd = A.to(cuda), W.to(cuda), bias.to(cuda)      # alive until the kernel has run
    _lib.check(L.mk_gemm_tc_groups(G, gs, M, N, K, _p(Ad), K, 1, _p(Wd), 1, K, _p(C), N, _p(bd),
                                   BIAS | RELU, None, 0, None, 0, None, None,
                                   engine._stream_handle()))
    engine.sync()
    for g in range(G):
        ref = torch.relu(A.double() @ W[g].double().T + bias[g].double())
        assert float((C[g].cpu().double() - ref).abs().max()) <= _tol(ref, K), g
    # G^T X per group, K = 900 rows: split K
    Kb = 900
    Gm = torch.tensor(rng.standard_normal((G, Kb, 64)), dtype=torch.float32).bfloat16()
    X = torch.tensor(rng.standard_normal((G, Kb, 48)), dtype=torch.float32).bfloat16()
    E = torch.full((G, 64, 48), float("nan"), dtype=torch.float32, device=cuda)
    gs = (ctypes.c_longlong * 6)(Kb * 64, Kb * 48, 64 * 48, 0, 0, 0)
    Gd, Xd = Gm.to(cuda), X.to(cuda)
    _lib.check(L.mk_gemm_tc_groups(G, gs, 64, 48, Kb, _p(Gd), 1, 64, _p(Xd), 48, 1, _p(E), 48,
                                   None, 0, None, 0, None, 0, None, None, engine._stream_handle()))
    engine.sync()
    for g in range(G):
        ref = Gm[g].double().T @ X[g].double()
        assert float((E[g].cpu().double() - ref).abs().max()) <= _tol(ref, Kb), g
