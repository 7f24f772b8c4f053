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


@pytest.mark.parametrize("weighted", [False, True])
def test_mlp_gradients_match_oracle(cuda, weighted):
    rng = np.random.default_rng(1)
    net = MLP(24, 96, hidden=64, n_hidden=3, seed=2, device=cuda)
    X = torch.tensor(omlp.bf16(rng.standard_normal((50, 24))), dtype=torch.bfloat16, device=cuda)
    T = torch.tensor(rng.standard_normal((50, 96)), dtype=torch.float32, device=cuda)
    w = rng.uniform(0.1, 10.0, 96).astype(np.float32) if weighted else None
    acts, posts, Y = net.forward(X)
    loss, G, Gb = net.mse(Y, T, torch.tensor(w, device=cuda) if weighted else None)
    dW, db = net.backward(acts, posts, G, Gb)
    Ws = [w_.float().cpu().numpy() for w_ in net.Wb]
    bs = [b.cpu().numpy() for b in net.b]
    H, oposts, oY = omlp.forward(X.float().cpu().numpy(), Ws, bs)
    odW, odb, oloss = omlp.backward(H, oposts, oY, T.cpu().numpy(), Ws, col_w=w)
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


def test_graph_captured_training_matches_eager(cuda):
    """fit_graph (one captured step replayed, step and learning rate in device
    memory) trains the same network as the eager loop."""
    rng = np.random.default_rng(4)
    X = torch.tensor(omlp.bf16(rng.standard_normal((40, 24))), dtype=torch.bfloat16, device=cuda)
    T = torch.tensor(rng.standard_normal((40, 9)), dtype=torch.float32, device=cuda)
    w = torch.tensor(rng.uniform(0.5, 2.0, 9), dtype=torch.float32, device=cuda)
    a = MLP(24, 9, hidden=32, n_hidden=2, seed=3, device=cuda)
    b = MLP(24, 9, hidden=32, n_hidden=2, seed=3, device=cuda)
    la = a.fit(X, T, steps=60, lr=3e-3, col_w=w)
    lb = b.fit_graph(X, T, steps=60, lr=3e-3, col_w=w)
    assert a.steps == b.steps == 60
    for wa, wb in zip(a.W + a.b, b.W + b.b):
        assert torch.allclose(wa, wb, rtol=1e-4, atol=1e-6), float((wa - wb).abs().max())
    assert abs(float(la[-1]) - float(lb[-1])) <= 1e-4 * abs(float(la[-1])) + 1e-7
    # continuing (the refinement step) keeps the Adam step count
    b.fit_graph(X, T, steps=10, lr=1e-3, col_w=w)
    assert b.steps == 70


def test_frame_basis_decode_on_the_gemm(cuda):
    """Principal components of a set of frames and their decoding through
    the BF16 GEMM with hi/lo splitting: full rank reproduces the frames."""
    rng = np.random.default_rng(5)
    X = torch.tensor(rng.random((40, 300)), dtype=torch.float32, device=cuda)
    basis = surrogate.FrameBasis(X, 64)
    assert basis.rank == 39          # 40 centred frames span 39 dimensions
    VV = (basis.V @ basis.V.T).cpu().numpy()
    assert np.allclose(VV, np.eye(39), atol=1e-4)
    net = MLP(4, 4, hidden=8, n_hidden=1, device=cuda)
    Xr = basis.decode(net, basis.coefficients(X).contiguous())
    assert float((Xr - X).abs().max()) < 1e-4


def test_surrogate_scan_gains_over_exact(cuda):
    """A small strained crystal (2.05M atoms), 49 x 49 theta x chi grid over
    +-0.2 deg, 64 x 64 ROI: exact training frames every 4th point per axis
    (169 = a 13 x 13 grid), the spline + network prediction for the rest,
    every 8th predicted frame judged. Every frame is also computed exactly
    (timed: the exact-only scan), so the error of every returned frame, of
    the prediction alone and of the spline alone, and the gain, are all
    measured."""
    w = workloads.cu_bumps_scan_4m(cells=80, npix=128)
    th = np.radians(np.linspace(-0.2, 0.2, 49))
    ch = np.radians(np.linspace(-0.2, 0.2, 49))
    sc = SurrogateScan(w.beam, w.sample, w.detector, w.stage, th, ch, roi=64, stride=4,
                       judge_every=8, tol=0.02, sc_kwargs=w.sc_kwargs)
    res = sc.run(exact_all=True)
    me, fe, be = res["model_err"], res["final_err"], res["base_err"]
    pct = lambda x: np.percentile(x, [50, 90, 100])
    print({k: v for k, v in res.items() if k not in ("frames", "judge_err", "judge_err_base",
                                                      "model_err", "final_err", "base_err")},
          "prediction err pct 50/90/100", pct(me), "spline-only", pct(be),
          "judged held out", pct(res["judge_err"]), "spline-only", pct(res["judge_err_base"]))
    assert res["n_train"] == 169 and res["n_frames"] == 2401 and res["exact_measured"]
    assert np.isfinite(me).all() and torch.isfinite(res["frames"]).all()
    # every returned frame within the tolerance, and the prediction alone too
    assert fe.max() <= 0.02 and me.max() <= 0.02
    # the network adds to the spline on the frames it did not train on
    assert np.percentile(res["judge_err"], 90) < np.percentile(res["judge_err_base"], 90)
    assert res["n_fallback"] <= 7 * res["n_failed_judges"]
    # frames/s over the exact-only scan, both timed here
    assert res["gain"] > 1.5, res["gain"]



def test_grouped_networks_match_separate_ones(cuda):
    """A group of two networks (every launch serving both) computes what two
    separate networks with the same seeds compute on their own data: same
    initial weights, outputs, gradients, and the same weights after captured
    training."""
    rng = np.random.default_rng(8)
    X = torch.tensor(omlp.bf16(rng.standard_normal((2, 40, 24))), dtype=torch.bfloat16, device=cuda)
    T = torch.tensor(rng.standard_normal((2, 40, 16)), dtype=torch.float32, device=cuda)
    w = torch.tensor(rng.uniform(0.5, 2.0, 16), dtype=torch.float32, device=cuda)
    grp = MLP(24, 16, hidden=32, n_hidden=2, seed=5, device=cuda, groups=2)
    sep = [MLP(24, 16, hidden=32, n_hidden=2, seed=5 + g, device=cuda) for g in range(2)]
    for l in range(len(sep[0].W)):
        for g in range(2):
            assert torch.equal(grp.W[l][g], sep[g].W[l])
    acts, posts, Y = grp.forward(X)
    loss, G, Gb = grp.mse(Y, T, w)
    dW, db = grp.backward(acts, posts, G, Gb)
    losses = []
    for g in range(2):
        a, p, y = sep[g].forward(X[g].contiguous())
        assert torch.allclose(Y[g], y, rtol=1e-6, atol=1e-6)
        l_, G_, Gb_ = sep[g].mse(y, T[g].contiguous(), w)
        losses.append(float(l_))
        dW_, db_ = sep[g].backward(a, p, G_, Gb_)
        for l in range(len(dW_)):
            assert torch.allclose(dW[l][g], dW_[l], rtol=1e-5, atol=1e-7), (g, l)
            assert torch.allclose(db[l][g], db_[l], rtol=1e-5, atol=1e-7), (g, l)
    assert abs(float(loss) - sum(losses)) <= 1e-5 * sum(losses)
    grp.fit_graph(X, T, steps=30, lr=3e-3, col_w=w)
    for g in range(2):
        sep[g].fit_graph(X[g].contiguous(), T[g].contiguous(), steps=30, lr=3e-3, col_w=w)
        for l in range(len(sep[g].W)):
            assert torch.allclose(grp.W[l][g], sep[g].W[l], rtol=1e-4, atol=1e-6), (g, l)
    Yp = grp.predict(X[0].contiguous())
    assert Yp.shape == (2, 40, 16)
    assert torch.allclose(Yp[1], sep[1].predict(X[0].contiguous()), rtol=1e-5, atol=1e-6)
