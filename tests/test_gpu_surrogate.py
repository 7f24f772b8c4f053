"""Scan surrogate: the BF16 MLP kernels against an FP32/FP64 CPU reference,
its gradients against the oracle, and the surrogate-assisted scan against the
exact batched scan it replaces."""
import numpy as np
import pytest
import torch

from oracle import mlp as omlp
from mosaic_gb300 import surrogate, workloads
from mosaic_gb300.surrogate import MLP, SurrogateScan

pytestmark = pytest.mark.gpu


def _bf(x):
    return torch.as_tensor(omlp.bf16(x), dtype=torch.float32)


@pytest.mark.parametrize("M,N,K", [(37, 70, 45), (64, 64, 32), (130, 17, 300)])
def test_gemm_layouts_match_fp32_reference(cuda, M, N, K):
    """Forward (X W^T), input-gradient (G W) and weight-gradient (G^T X)
    layouts, ragged sizes, bias + ReLU epilogue, accumulate."""
    rng = np.random.default_rng(M * N + K)
    net = MLP(4, 4, hidden=8, n_hidden=1, device=cuda)       # for its GEMM wrapper
    A = _bf(rng.standard_normal((M, K)))
    W = _bf(rng.standard_normal((N, K)))
    bias = torch.tensor(rng.standard_normal(N), dtype=torch.float32)
    Ad, Wd = A.to(cuda).bfloat16(), W.to(cuda).bfloat16()
    C = torch.empty((M, N), dtype=torch.float32, device=cuda)
    Cb = torch.empty((M, N), dtype=torch.bfloat16, device=cuda)
    net._gemm(M, N, K, Ad, K, 1, Wd, 1, K, C, N, bias.to(cuda), surrogate.GEMM_BIAS | surrogate.GEMM_RELU, Cb, N)
    ref = torch.relu(A.double() @ W.double().T + bias.double())
    assert torch.allclose(C.cpu().double(), ref, rtol=1e-5, atol=1e-4 * float(ref.abs().max()))
    assert torch.allclose(Cb.cpu().double(), ref, rtol=1e-2, atol=1e-2 * float(ref.abs().max()))
    # G (M, N) @ W (N, K) -> (M, K), accumulated onto a preset C
    G = _bf(rng.standard_normal((M, N)))
    Gd = G.to(cuda).bfloat16()
    D = torch.full((M, K), 0.5, dtype=torch.float32, device=cuda)
    net._gemm(M, K, N, Gd, N, 1, Wd, K, 1, D, K, None, surrogate.GEMM_ACC, None, 0)
    assert torch.allclose(D.cpu().double(), G.double() @ W.double() + 0.5, rtol=1e-5, atol=1e-3)
    # G^T (N, M) @ A (M, K) -> (N, K)
    E = torch.empty((N, K), dtype=torch.float32, device=cuda)
    net._gemm(N, K, M, Gd, 1, N, Ad, K, 1, E, K, None, 0, None, 0)
    assert torch.allclose(E.cpu().double(), G.double().T @ A.double(), rtol=1e-5, atol=1e-3)


def test_mlp_gradients_match_oracle(cuda):
    rng = np.random.default_rng(1)
    net = MLP(24, 96, hidden=64, n_hidden=3, seed=2, device=cuda)
    X = torch.tensor(omlp.bf16(rng.standard_normal((50, 24))), dtype=torch.bfloat16, device=cuda)
    T = torch.tensor(rng.standard_normal((50, 96)), dtype=torch.float32, device=cuda)
    acts, posts, Y = net.forward(X)
    loss, G, Gb = net.mse(Y, T)
    dW, db = net.backward(acts, posts, G, Gb)
    Ws = [w.float().cpu().numpy() for w in net.Wb]
    bs = [b.cpu().numpy() for b in net.b]
    H, oposts, oY = omlp.forward(X.float().cpu().numpy(), Ws, bs)
    odW, odb, oloss = omlp.backward(H, oposts, oY, T.cpu().numpy(), Ws)
    assert abs(float(loss) - oloss) <= 1e-4 * oloss
    assert np.allclose(Y.cpu().numpy(), oY, rtol=1e-3, atol=1e-3 * np.abs(oY).max())
    for l in range(len(Ws)):
        g, o = dW[l].cpu().numpy().ravel(), odW[l].ravel()
        cos = float(g @ o / (np.linalg.norm(g) * np.linalg.norm(o)))
        assert cos > 0.9999, (l, cos)
        assert np.abs(g - o).max() <= 2e-2 * np.abs(o).max(), l
        assert np.allclose(db[l].cpu().numpy(), odb[l], rtol=1e-3, atol=1e-3 * np.abs(odb[l]).max())


def test_mlp_fits_a_smooth_field(cuda):
    xy = np.stack(np.meshgrid(np.linspace(-1, 1, 12), np.linspace(-1, 1, 12), indexing="ij"), -1).reshape(-1, 2)
    target = np.stack([np.sin(3 * xy[:, 0]) * np.cos(2 * xy[:, 1]) + k * 0.1 for k in range(40)], 1)
    feats = surrogate.fourier_features(xy, 8, cuda, f_max=1.5)
    net = MLP(feats.shape[1], 40, hidden=64, n_hidden=2, seed=0, device=cuda)
    T = torch.tensor(target, dtype=torch.float32, device=cuda)
    losses = net.fit(feats, T, steps=600, lr=3e-3)
    assert losses[-1] < 0.05 * losses[0]
    assert float(((net.predict(feats) - T) ** 2).mean()) < 2e-2


def test_surrogate_scan_gains_over_exact(cuda):
    """A small strained crystal, 25 x 25 theta x chi grid: exact training
    frames every 4th point per axis, the MLP for the rest, every 8th predicted
    frame re-judged. The surrogate-assisted scan must beat the exact batched
    scan in frames/s and keep judged frames within the 2% budget or send them
    (and their blocks) to the exact sum."""
    w = workloads.cu_bumps_scan_4m(cells=80, npix=128)      # 2.05M atoms
    th = np.radians(np.linspace(-0.2, 0.2, 49))
    ch = np.radians(np.linspace(-0.2, 0.2, 49))
    sc = SurrogateScan(w.beam, w.sample, w.detector, w.stage, th, ch, roi=64, stride=4,
                       judge_every=8, tol=0.02, hidden=256, n_hidden=4, n_freq=16, fit_steps=1000,
                       sc_kwargs=w.sc_kwargs)
    res = sc.run(verify=16)
    print({k: v for k, v in res.items() if k not in ("frames", "judge_err", "verify_err")},
          "judge err median", float(np.median(res["judge_err"])),
          "verify err median", float(np.median(res["verify_err"])) if len(res["verify_err"]) else None)
    assert res["n_train"] == 169 and res["n_frames"] == 2401
    assert res["final_loss"] < 0.2
    assert np.isfinite(res["judge_err"]).all() and np.isfinite(res["verify_err"]).all()
    # frames whose judge failed were replaced by the exact sum
    assert res["n_fallback"] <= 7 * res["n_failed_judges"]
    assert torch.isfinite(res["frames"]).all()
    # what the trained network gains over computing every frame exactly
    assert res["exact_frames"] < res["n_frames"]
    assert res["gain"] > 1.0, res["gain"]
