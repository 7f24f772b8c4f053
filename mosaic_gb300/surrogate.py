"""Learned scan surrogate: a BF16 MLP that predicts intermediate scan frames.

For a 2-D motor scan (theta x chi) the exact kinematic sum is computed on a
sub-grid of training frames (every ``stride``-th point along each axis) in
one batched launch; an MLP maps the two motor coordinates (with Fourier
features) to the log-intensity of every ROI pixel and predicts the other
frames. Every ``judge_every``-th predicted frame is recomputed exactly; if its
relative error max|I_pred - I| / max I exceeds ``tol`` it falls back to the
exact sum, together with the predicted frames it stands for.

The network trains and predicts on the GPU with the library's own kernels
(``mk_gemm_bf16``: BF16 operands, FP32 accumulation on the tensor cores;
``mk_adam`` on FP32 master weights; ``mk_fourier_features``, ``mk_mse``,
``mk_relu_backward``, ``mk_bias_grad``). No counterpart in the reference: the
reference runs one full exposure per scan step (Experiment.py:285-336).
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
import torch

from . import _lib, engine
from ._lib import check
from .scan import BatchedScan, frames_from_motors

GEMM_ACC, GEMM_BIAS, GEMM_RELU = 1, 2, 4


def _p(t):
    return t.data_ptr() if t is not None else None


class MLP:
    """Fully connected ReLU network, BF16 weights (FP32 masters), FP32 accumulation."""

    def __init__(self, n_in, n_out, hidden=256, n_hidden=4, seed=0, device="cuda"):
        self.L = engine._require_cuda()
        self.dev = torch.device(device)
        self.dims = [int(n_in)] + [int(hidden)] * int(n_hidden) + [int(n_out)]
        rng = np.random.default_rng(seed)
        self.W, self.Wb, self.b, self.mW, self.vW, self.mb, self.vb = [], [], [], [], [], [], []
        for l in range(len(self.dims) - 1):
            K, N = self.dims[l], self.dims[l + 1]
            last = l == len(self.dims) - 2
            std = np.sqrt((1.0 if last else 2.0) / K)
            W = torch.tensor(rng.standard_normal((N, K)) * std, dtype=torch.float32, device=self.dev)
            self.W.append(W)
            self.Wb.append(W.to(torch.bfloat16))
            self.b.append(torch.zeros(N, dtype=torch.float32, device=self.dev))
            self.mW.append(torch.zeros_like(W))
            self.vW.append(torch.zeros_like(W))
            self.mb.append(torch.zeros(N, dtype=torch.float32, device=self.dev))
            self.vb.append(torch.zeros(N, dtype=torch.float32, device=self.dev))
        self.steps = 0

    @property
    def n_params(self):
        return sum(w.numel() + b.numel() for w, b in zip(self.W, self.b))

    def _gemm(self, M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, bias, flags, Cb, ldcb):
        check(self.L.mk_gemm_bf16(M, N, K, _p(A), sam, sak, _p(B), sbk, sbn, _p(C), ldc, _p(bias),
                                  flags, _p(Cb), ldcb, engine._stream_handle()))

    def forward(self, X):
        """X (B, n_in) bf16 -> (layer inputs (bf16), hidden post-activations (f32), Y (f32))."""
        B = int(X.shape[0])
        acts, posts = [X], []
        Y = None
        for l in range(len(self.dims) - 1):
            K, N = self.dims[l], self.dims[l + 1]
            last = l == len(self.dims) - 2
            C = torch.empty((B, N), dtype=torch.float32, device=self.dev)
            Cb = None if last else torch.empty((B, N), dtype=torch.bfloat16, device=self.dev)
            self._gemm(B, N, K, acts[-1], K, 1, self.Wb[l], 1, K, C, N, self.b[l],
                       GEMM_BIAS | (0 if last else GEMM_RELU), Cb, N)
            if last:
                Y = C
            else:
                posts.append(C)
                acts.append(Cb)
        return acts, posts, Y

    def backward(self, acts, posts, G, Gb):
        """Gradients of the loss given dL/dY (f32 G and its bf16 copy Gb)."""
        B = int(G.shape[0])
        dW, db = [None] * len(self.W), [None] * len(self.W)
        for l in range(len(self.dims) - 2, -1, -1):
            K, N = self.dims[l], self.dims[l + 1]
            dW[l] = torch.empty((N, K), dtype=torch.float32, device=self.dev)
            self._gemm(N, K, B, Gb, 1, N, acts[l], K, 1, dW[l], K, None, 0, None, 0)
            db[l] = torch.empty(N, dtype=torch.float32, device=self.dev)
            check(self.L.mk_bias_grad(B, N, _p(G), _p(db[l]), engine._stream_handle()))
            if l == 0:
                break
            dH = torch.empty((B, K), dtype=torch.float32, device=self.dev)
            self._gemm(B, K, N, Gb, N, 1, self.Wb[l], K, 1, dH, K, None, 0, None, 0)
            G = torch.empty((B, K), dtype=torch.float32, device=self.dev)
            Gb = torch.empty((B, K), dtype=torch.bfloat16, device=self.dev)
            check(self.L.mk_relu_backward(B * K, _p(dH), _p(posts[l - 1]), _p(G), _p(Gb),
                                          engine._stream_handle()))
        return dW, db

    def mse(self, Y, T):
        """(loss as a device scalar, dL/dY f32, bf16)."""
        n = Y.numel()
        G = torch.empty_like(Y)
        Gb = torch.empty(Y.shape, dtype=torch.bfloat16, device=self.dev)
        part = torch.empty((n + 255) // 256, dtype=torch.float64, device=self.dev)
        check(self.L.mk_mse(n, _p(Y), _p(T), _p(G), _p(Gb), _p(part), engine._stream_handle()))
        return part.sum() / n, G, Gb

    def adam(self, dW, db, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        self.steps += 1
        sh = engine._stream_handle()
        for l in range(len(self.W)):
            check(self.L.mk_adam(self.W[l].numel(), _p(self.W[l]), _p(dW[l]), _p(self.mW[l]),
                                 _p(self.vW[l]), _p(self.Wb[l]), lr, beta1, beta2, eps, self.steps,
                                 weight_decay, sh))
            check(self.L.mk_adam(self.b[l].numel(), _p(self.b[l]), _p(db[l]), _p(self.mb[l]),
                                 _p(self.vb[l]), None, lr, beta1, beta2, eps, self.steps, 0.0, sh))

    def fit(self, X, T, steps=1500, lr=2e-3, lr_final=1e-4, batch=None, seed=0):
        """Adam on mean squared error; cosine learning-rate decay. Returns the loss history."""
        gen = torch.Generator(device=self.dev)
        gen.manual_seed(seed)
        n = int(X.shape[0])
        losses = []
        for s in range(steps):
            a = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * s / max(steps - 1, 1)))
            if batch and batch < n:
                idx = torch.randperm(n, generator=gen, device=self.dev)[:batch]
                Xb, Tb = X[idx], T[idx]
            else:
                Xb, Tb = X, T
            acts, posts, Y = self.forward(Xb)
            loss, G, Gb = self.mse(Y, Tb)
            dW, db = self.backward(acts, posts, G, Gb)
            self.adam(dW, db, float(a))
            losses.append(loss)
        return torch.stack(losses).cpu().numpy()

    def predict(self, X, chunk=4096):
        outs = []
        for i in range(0, int(X.shape[0]), chunk):
            outs.append(self.forward(X[i:i + chunk])[2])
        return torch.cat(outs)


def fourier_features(xy, n_freq=16, device="cuda", f_max=4.0, f_min=0.25):
    """(n, 2) coordinates in [-1, 1] -> (n, width) bf16 network inputs with
    ``n_freq`` frequencies geometrically spaced from f_min to f_max cycles per
    unit. f_max must stay below the Nyquist limit of the training grid
    (n_train_per_axis / 4 cycles per unit): higher features only alias
    between training frames."""
    L = engine._require_cuda()
    xy = torch.as_tensor(np.ascontiguousarray(xy, dtype=np.float32)).to(device)
    width = 2 + 4 * int(n_freq)
    width = (width + 7) // 8 * 8
    ratio = (f_max / f_min) ** (1.0 / max(int(n_freq) - 1, 1)) if n_freq > 1 else 1.0
    out = torch.empty((int(xy.shape[0]), width), dtype=torch.bfloat16, device=device)
    check(L.mk_fourier_features(int(xy.shape[0]), _p(xy), int(n_freq), float(f_min),
                                float(max(ratio, 1.0)), width, _p(out), engine._stream_handle()))
    return out


def frame_rel_error(I_pred, I_exact):
    """max over pixels |I_pred - I| / max I, per frame (rows)."""
    num = (I_pred - I_exact).abs().amax(dim=1)
    return num / I_exact.amax(dim=1).clamp_min(1e-300)


class SurrogateScan:
    """Surrogate-assisted theta x chi scan (see the module docstring).

    Args:
        beam, sample, detector, stage: as for BatchedScan / scan_nD.
        theta, chi: offsets [rad] added to the stage's mu and chi motors.
        roi: square ROI side (pixels) around the detector centre.
        stride: training frames every ``stride`` points along each axis
            (``raster=True``: every ``stride``-th frame in raster order).
        judge_every, tol: exact re-judging cadence and fallback threshold.
    """

    def __init__(self, beam, sample, detector, stage, theta, chi, roi=128, stride=4, raster=False,
                 judge_every=8, tol=0.02, hidden=256, n_hidden=4, n_freq=16, fit_steps=1500,
                 lr=2e-3, seed=0, sc_kwargs=None, device="cuda"):
        self.beam, self.sample, self.detector, self.stage = beam, sample, detector, stage
        self.theta = np.asarray(theta, dtype=np.float64)
        self.chi = np.asarray(chi, dtype=np.float64)
        self.roi, self.stride, self.raster = int(roi), int(stride), bool(raster)
        self.judge_every, self.tol = int(judge_every), float(tol)
        self.hidden, self.n_hidden, self.n_freq = hidden, n_hidden, n_freq
        self.fit_steps, self.lr, self.seed = fit_steps, lr, seed
        self.kw = dict(apply_polarization=False, spherical_decay=False, remove_forward=False)
        self.kw.update(sc_kwargs or {})
        self.dev = torch.device(device)
        nt, nc = len(self.theta), len(self.chi)
        ii, jj = np.meshgrid(np.arange(nt), np.arange(nc), indexing="ij")
        self.ij = np.stack([ii.ravel(), jj.ravel()], 1)          # raster order
        norm = lambda v, n: (2.0 * v / max(n - 1, 1)) - 1.0
        self.xy = np.stack([norm(self.ij[:, 0], nt), norm(self.ij[:, 1], nc)], 1)
        if self.raster:
            self.train = np.arange(len(self.ij)) % self.stride == 0
        else:
            self.train = (self.ij[:, 0] % self.stride == 0) & (self.ij[:, 1] % self.stride == 0)
        mu0 = float(stage.motor_value[stage.motor_index("mu")])
        chi0 = float(stage.motor_value[stage.motor_index("chi")])
        self.steps = [dict(mu=mu0 + self.theta[i], chi=chi0 + self.chi[j]) for i, j in self.ij]
        self._staged = None

    def exact(self, idx):
        """Exact intensities (len(idx), roi*roi) of the given frames, one batched launch."""
        idx = np.asarray(idx)
        if idx.size == 0:
            return torch.zeros((0, self.roi * self.roi), dtype=torch.float32, device=self.dev)
        frames = frames_from_motors(self.stage, self.detector, [self.steps[i] for i in idx],
                                    [self.roi] * len(idx))
        if len(frames) == 1:               # a one-frame batch still goes through the scan path
            frames = frames * 2
        scan = BatchedScan(self.beam, self.sample, frames, staged=self._staged, **self.kw)
        self._staged = self._staged or scan
        out, _ = scan.run()
        I = (out * out).sum(1).reshape(len(frames), -1)[: len(idx)].float()
        return I

    def run(self, verify=0):
        """Run the scan; ``verify`` > 0 also computes exact frames for that many
        unjudged predicted frames (not timed) to measure the true error."""
        sync = torch.cuda.synchronize
        n = len(self.ij)
        t = {}
        sync()
        t0 = time.perf_counter()
        tr = np.flatnonzero(self.train)
        I_train = self.exact(tr)
        sync()
        t["exact_train"] = time.perf_counter() - t0
        # targets: per-pixel standardised log intensity
        eps = 1e-6 * float(I_train.max())
        logI = torch.log(I_train + eps)
        mu, sd = logI.mean(0, keepdim=True), logI.std(0, keepdim=True).clamp_min(1e-3)
        T = ((logI - mu) / sd).contiguous()
        # highest feature frequency: half the Nyquist limit of the training grid
        n_axis = min(len(np.unique(self.ij[tr, 0])), len(np.unique(self.ij[tr, 1])))
        feats = fourier_features(self.xy, self.n_freq, self.dev, f_max=max(0.5, n_axis / 8.0))
        t0 = time.perf_counter()
        self.net = MLP(feats.shape[1], T.shape[1], self.hidden, self.n_hidden, self.seed, self.dev)
        self.losses = self.net.fit(feats[torch.as_tensor(tr, device=self.dev)], T,
                                   steps=self.fit_steps, lr=self.lr)
        sync()
        t["fit"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        pred_idx = np.flatnonzero(~self.train)
        Yp = self.net.predict(feats[torch.as_tensor(pred_idx, device=self.dev)])
        I_pred = (torch.exp(Yp * sd + mu) - eps).clamp_min(0.0)
        sync()
        t["predict"] = time.perf_counter() - t0
        # judge every judge_every-th predicted frame; a failed judge sends its
        # block of predicted frames to the exact sum
        blocks = [np.arange(b, min(b + self.judge_every, len(pred_idx)))
                  for b in range(0, len(pred_idx), self.judge_every)]
        judged = np.array([blk[0] for blk in blocks], dtype=np.int64)
        t0 = time.perf_counter()
        I_j = self.exact(pred_idx[judged])
        err_j = frame_rel_error(I_pred[judged], I_j).cpu().numpy()
        sync()
        t["judge"] = time.perf_counter() - t0
        I_pred[torch.as_tensor(judged, device=self.dev)] = I_j
        failed = [blk for blk, e in zip(blocks, err_j) if e > self.tol]
        fb = np.concatenate([blk[1:] for blk in failed]) if failed else np.zeros(0, np.int64)
        t0 = time.perf_counter()
        if fb.size:
            I_pred[torch.as_tensor(fb, device=self.dev)] = self.exact(pred_idx[fb])
        sync()
        t["fallback"] = time.perf_counter() - t0
        frames = torch.empty((n, self.roi * self.roi), dtype=torch.float32, device=self.dev)
        frames[torch.as_tensor(tr, device=self.dev)] = I_train
        frames[torch.as_tensor(pred_idx, device=self.dev)] = I_pred
        exact_frames = len(tr) + len(judged) + int(fb.size)
        total = sum(t.values())
        per_exact = t["exact_train"] / max(len(tr), 1)
        res = dict(frames=frames, n_frames=n, n_train=len(tr), n_judged=len(judged),
                   n_fallback=int(fb.size), n_failed_judges=len(failed), exact_frames=exact_frames,
                   judge_err=err_j, times=t, seconds=total, frames_per_s=n / total,
                   exact_frames_per_s=1.0 / per_exact, exact_scan_seconds_est=n * per_exact,
                   gain=(n * per_exact) / total, final_loss=float(self.losses[-1]),
                   params=self.net.n_params)
        if verify:
            rng = np.random.default_rng(self.seed + 1)
            unjudged = np.setdiff1d(np.arange(len(pred_idx)), np.concatenate([judged, fb]))
            pick = rng.choice(unjudged, size=min(int(verify), unjudged.size), replace=False) \
                if unjudged.size else np.zeros(0, np.int64)
            I_true = self.exact(pred_idx[pick])
            res["verify_err"] = frame_rel_error(I_pred[torch.as_tensor(pick, device=self.dev)],
                                                I_true).cpu().numpy()
        return res
