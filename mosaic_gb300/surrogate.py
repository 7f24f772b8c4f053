"""Learned scan surrogate: a BF16 MLP that predicts intermediate scan frames.

For a 2-D motor scan (theta x chi) the exact kinematic sum is computed on a
grid of training frames (every ``stride``-th point along each axis) and on
the judged frames, in one batched launch. Each frame is described by the
principal-component coefficients of its peak-normalised intensity I / max I
(``FrameBasis``, from the training frames) and the log of its peak. The
prediction of a frame is the interpolating bicubic spline of the training
frames' descriptions over the motor grid plus a correction that an MLP
(Fourier features of the two motor coordinates, ReLU layers, BF16 weights
and activations, FP32 accumulation) learns: the spline's residual, which is
zero at the training frames and measured at the judged ones. Every
``judge_every``-th predicted frame is judged: its exact frame is compared
with the prediction, and if the relative error max|I_pred - I| / max I
exceeds ``tol``, the rest of its block of frames falls back to the exact
sum. Two networks are trained, each on the judged frames of alternate
blocks, so that every judged frame is predicted by the network that never
saw it; the other frames take the mean of the two. The judged frames'
errors with and without the network measure, held out, what the network
adds to the spline.

Why this form (measured on the 101 x 101 scan of the 4M-atom strained
crystal, every frame also computed exactly): a network alone, fed the motor
coordinates, fits even its own training frames only to ~2 % and missed 2 %
on ~1 % of the frames it predicted; the spline alone stays within 0.5 %;
the network trained on the spline's residual brings the 90th percentile of
the held-out judged frames' error from 6e-4 to ~2e-4.

The network trains and predicts on the GPU with the library's own kernels
(``mk_gemm_bf16``: BF16 operands, FP32 accumulation on the tensor cores;
``mk_adam_sched`` on FP32 master weights; ``mk_fourier_features``,
``mk_mse_weighted``, ``mk_relu_backward``, ``mk_bias_grad``); the frames are
decoded from their descriptions on ``mk_gemm_bf16`` too. No counterpart in
the reference: the reference runs one full exposure per scan step
(Experiment.py:285-336).
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
    """Fully connected ReLU network, BF16 weights (FP32 masters), FP32
    accumulation; ``groups`` independent networks of the same shape trained
    and evaluated together (every GEMM and bias-gradient launch serves all
    of them: grid z = network). All parameters live in one flat FP32 buffer
    (with its BF16 copy, Adam moments and gradient), so one Adam launch
    updates them all; ``W[l]`` (N, K) and ``b[l]`` (N) are views into it,
    with a leading group axis when groups > 1."""

    def __init__(self, n_in, n_out, hidden=256, n_hidden=4, seed=0, device="cuda", groups=1):
        self.L = engine._require_cuda()
        self.dev = torch.device(device)
        self.G = int(groups)
        self.dims = [int(n_in)] + [int(hidden)] * int(n_hidden) + [int(n_out)]
        shapes = [(self.dims[l + 1], self.dims[l]) for l in range(len(self.dims) - 1)]
        nl = len(shapes)
        pad8 = lambda n: (n + 7) // 8 * 8      # 16-byte boundaries of the bf16 copy
        self._wpad = [pad8(N * K) for N, K in shapes]
        self._bpad = [pad8(N) for N, _ in shapes]
        offs, o = [], 0
        for n in self._wpad + self._bpad:      # layer blocks of G networks each
            offs.append(o)
            o += self.G * n
        total = o
        f32 = dict(dtype=torch.float32, device=self.dev)
        self.P = torch.zeros(total, **f32)
        self.Pb = torch.zeros(total, dtype=torch.bfloat16, device=self.dev)
        self.mP, self.vP, self.gP = (torch.zeros(total, **f32) for _ in range(3))
        G = self.G

        def view(buf, i, shape, gstride):
            if G == 1:
                return buf[offs[i]: offs[i] + int(np.prod(shape))].view(*shape)
            st = [gstride] + [int(np.prod(shape[j + 1:])) for j in range(len(shape))]
            return torch.as_strided(buf, (G,) + tuple(shape), st, offs[i])

        self.W = [view(self.P, l, shapes[l], self._wpad[l]) for l in range(nl)]
        self.Wb = [view(self.Pb, l, shapes[l], self._wpad[l]) for l in range(nl)]
        self.b = [view(self.P, nl + l, (shapes[l][0],), self._bpad[l]) for l in range(nl)]
        self.dW = [view(self.gP, l, shapes[l], self._wpad[l]) for l in range(nl)]
        self.db = [view(self.gP, nl + l, (shapes[l][0],), self._bpad[l]) for l in range(nl)]
        for g in range(G):
            rng = np.random.default_rng(seed + g)
            for l, (N, K) in enumerate(shapes):
                std = np.sqrt((1.0 if l == nl - 1 else 2.0) / K)
                w = self.W[l] if G == 1 else self.W[l][g]
                w.copy_(torch.tensor(rng.standard_normal((N, K)) * std, **f32))
        self.Pb.copy_(self.P.to(torch.bfloat16))
        self.steps = 0

    @property
    def n_params(self):
        """Parameters of one network of the group."""
        return sum(w[0].numel() + b[0].numel() if self.G > 1 else w.numel() + b.numel()
                   for w, b in zip(self.W, self.b))

    def _gemm(self, M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, bias, flags, Cb, ldcb, mask=None,
              ldm=0, row_scale=None, row_map=None, gstrides=None):
        """C (+)= A B on the tcgen05 GEMM, fused epilogue; ``gstrides`` (A, B,
        C, Cb, bias, mask element strides) runs the G networks' products in
        one launch."""
        if gstrides is None or self.G == 1:
            check(self.L.mk_gemm_tc(M, N, K, _p(A), sam, sak, _p(B), sbk, sbn, _p(C), ldc, _p(bias),
                                    flags, _p(Cb), ldcb, _p(mask), ldm, _p(row_scale), _p(row_map),
                                    engine._stream_handle()))
        else:
            gs = (ctypes.c_longlong * 6)(*[int(v) for v in gstrides])
            check(self.L.mk_gemm_tc_groups(self.G, gs, M, N, K, _p(A), sam, sak, _p(B), sbk, sbn,
                                           _p(C), ldc, _p(bias), flags, _p(Cb), ldcb, _p(mask), ldm,
                                           None, None, engine._stream_handle()))

    def _new(self, B, N, dtype):
        shape = (B, N) if self.G == 1 else (self.G, B, N)
        return torch.empty(shape, dtype=dtype, device=self.dev)

    def forward(self, X):
        """X (B, n_in) bf16 -- shared by the G networks -- or (G, B, n_in) ->
        (layer inputs (bf16), hidden post-activations (f32), Y (f32)), each
        with a leading group axis when G > 1."""
        B = int(X.shape[-2])
        shared = X.dim() == 2
        acts, posts = [X], []
        Y = None
        for l in range(len(self.dims) - 1):
            K, N = self.dims[l], self.dims[l + 1]
            last = l == len(self.dims) - 2
            C = self._new(B, N, torch.float32)
            Cb = None if last else self._new(B, N, torch.bfloat16)
            ga = 0 if (l == 0 and shared) else B * K
            self._gemm(B, N, K, acts[-1], K, 1, self.Wb[l], 1, K, C, N, self.b[l],
                       GEMM_BIAS | (0 if last else GEMM_RELU), Cb, N,
                       gstrides=(ga, self._wpad[l], B * N, B * N, self._bpad[l], 0))
            if last:
                Y = C
            else:
                posts.append(C)
                acts.append(Cb)
        return acts, posts, Y

    def backward(self, acts, posts, G, Gb):
        """Gradients of the loss given dL/dY (f32 G and its bf16 copy Gb),
        into the flat gradient buffer: returns its (dW, db) views. The input
        gradient of a hidden layer carries the ReLU derivative in its
        GEMM's epilogue (the layer's outputs as the mask)."""
        B = int(G.shape[-2])
        for l in range(len(self.dims) - 2, -1, -1):
            K, N = self.dims[l], self.dims[l + 1]
            gx = 0 if (l == 0 and acts[0].dim() == 2) else B * K
            self._gemm(N, K, B, Gb, 1, N, acts[l], K, 1, self.dW[l], K, None, 0, None, 0,
                       gstrides=(B * N, gx, self._wpad[l], 0, 0, 0))
            check(self.L.mk_bias_grad_groups(self.G, B, N, _p(G), B * N, _p(self.db[l]),
                                             self._bpad[l], engine._stream_handle()))
            if l == 0:
                break
            G2 = self._new(B, K, torch.float32)
            Gb2 = self._new(B, K, torch.bfloat16)
            self._gemm(B, K, N, Gb, N, 1, self.Wb[l], K, 1, G2, K, None, 0, Gb2, K,
                       mask=posts[l - 1], ldm=K,
                       gstrides=(B * N, self._wpad[l], B * K, B * K, 0, B * K))
            G, Gb = G2, Gb2
        return self.dW, self.db

    def mse(self, Y, T, col_w=None):
        """(loss as a device scalar, dL/dY f32, bf16); ``col_w`` weights the
        output columns (float32 device vector). With G networks the loss is
        the sum of theirs and each network's gradient is its own loss's."""
        n = Y.numel()
        G = torch.empty_like(Y)
        Gb = torch.empty(Y.shape, dtype=torch.bfloat16, device=self.dev)
        part = torch.empty((n + 255) // 256, dtype=torch.float64, device=self.dev)
        if col_w is None and self.G == 1:
            check(self.L.mk_mse(n, _p(Y), _p(T), _p(G), _p(Gb), _p(part), engine._stream_handle()))
        else:
            # 2 w (y - t) / n over all G networks' entries: weights times G
            # make each network's gradient that of its own mean
            w = (col_w if col_w is not None else torch.ones(Y.shape[-1], device=self.dev))
            if self.G > 1:
                w = (w * float(self.G)).contiguous()
            check(self.L.mk_mse_weighted(n, int(Y.shape[-1]), _p(Y), _p(T), _p(w), _p(G),
                                         _p(Gb), _p(part), engine._stream_handle()))
        return part.sum() / n, G, Gb

    def adam(self, dW, db, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        """One Adam step on every parameter (the gradients are the flat
        buffer's views that ``backward`` returned)."""
        self.steps += 1
        check(self.L.mk_adam(self.P.numel(), _p(self.P), _p(self.gP), _p(self.mP), _p(self.vP),
                             _p(self.Pb), lr, beta1, beta2, eps, self.steps, weight_decay,
                             engine._stream_handle()))

    def fit(self, X, T, steps=1500, lr=2e-3, lr_final=1e-4, batch=None, seed=0, col_w=None):
        """Adam on (column-weighted) mean squared error; cosine learning-rate
        decay. Returns the loss history."""
        gen = torch.Generator(device=self.dev)
        gen.manual_seed(seed)
        n = int(X.shape[-2])
        losses = []
        for s in range(steps):
            a = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * s / max(steps - 1, 1)))
            if batch and batch < n:
                idx = torch.randperm(n, generator=gen, device=self.dev)[:batch]
                Xb, Tb = X.index_select(-2, idx), T.index_select(-2, idx)
            else:
                Xb, Tb = X, T
            acts, posts, Y = self.forward(Xb)
            loss, G, Gb = self.mse(Y, Tb, col_w)
            dW, db = self.backward(acts, posts, G, Gb)
            self.adam(dW, db, float(a))
            losses.append(loss)
        return torch.stack(losses).cpu().numpy()

    def fit_graph(self, X, T, steps=1500, lr=2e-3, lr_final=1e-4, col_w=None):
        """``fit`` on the full batch with one training step (forward, loss,
        backward, Adam) captured as a CUDA graph and replayed ``steps`` times:
        the same arithmetic and cosine schedule, without a host round trip per
        step (the step number and learning rate live in device memory,
        mk_adam_sched). Returns the final loss (1-element array)."""
        return fit_graphs([self], [X], [T], steps, lr, lr_final, [col_w])[0]

    def _graph_state(self, steps, lr, lr_final):
        """Device-side schedule and step counter of a captured training run;
        makes the first call of its kernels outside the capture."""
        sh = engine._stream_handle
        sched = lr_final + 0.5 * (lr - lr_final) * (
            1 + np.cos(np.pi * np.arange(steps) / max(steps - 1, 1)))
        lr_d = torch.tensor(sched, dtype=torch.float32, device=self.dev)
        step0 = int(self.steps)
        counter = torch.tensor([step0], dtype=torch.int32, device=self.dev)
        tmp = torch.zeros(4, dtype=torch.float32, device=self.dev)
        check(self.L.mk_adam_sched(1, _p(tmp[0:]), _p(tmp[1:]), _p(tmp[2:]), _p(tmp[3:]), None,
                                   _p(lr_d), _p(counter), step0, 0.9, 0.999, 1e-8, 0.0, sh()))
        cnt2 = counter.clone()
        check(self.L.mk_counter_add(_p(cnt2), 1, sh()))
        return lr_d, counter, step0

    def _step(self, X, T, col_w, lr_d, counter, step0):
        """One training step on the current stream (captured): returns the
        loss as a device scalar."""
        acts, posts, Y = self.forward(X)
        loss, G, Gb = self.mse(Y, T, col_w)
        self.backward(acts, posts, G, Gb)
        s = engine._stream_handle()
        check(self.L.mk_adam_sched(self.P.numel(), _p(self.P), _p(self.gP), _p(self.mP),
                                   _p(self.vP), _p(self.Pb), _p(lr_d), _p(counter), step0,
                                   0.9, 0.999, 1e-8, 0.0, s))
        check(self.L.mk_counter_add(_p(counter), 1, s))
        return loss

    def predict(self, X, chunk=4096):
        """Outputs for inputs X (B, n_in): (B, n_out), or (G, B, n_out)."""
        outs = []
        for i in range(0, int(X.shape[0]), chunk):
            outs.append(self.forward(X[i:i + chunk])[2])
        return torch.cat(outs, dim=-2)


def fit_graphs(nets, Xs, Ts, steps=1500, lr=2e-3, lr_final=1e-4, col_ws=None):
    """Train independent networks together: one CUDA graph holds a training
    step of every network, each on its own stream (forked from and joined
    back to the current one), and is replayed ``steps`` times, so the
    networks' small kernels run side by side on the GPU. Per network the
    arithmetic is ``MLP.fit_graph``'s. Returns each network's final loss
    (1-element arrays)."""
    if steps <= 0:
        return [np.zeros(0) for _ in nets]
    col_ws = col_ws or [None] * len(nets)
    states = [net._graph_state(steps, lr, lr_final) for net in nets]
    dev = nets[0].dev
    torch.cuda.synchronize(dev)
    cur = torch.cuda.current_stream(dev)
    side = [torch.cuda.Stream(dev) for _ in nets[1:]]
    g = torch.cuda.CUDAGraph()
    losses = [None] * len(nets)
    with torch.cuda.graph(g):
        cap = torch.cuda.current_stream(dev)
        for i, net in enumerate(nets):
            st = cap if i == 0 else side[i - 1]
            if i:
                st.wait_stream(cap)
            with torch.cuda.stream(st):
                losses[i] = net._step(Xs[i], Ts[i], col_ws[i], *states[i])
        for st in side:
            cap.wait_stream(st)
    for _ in range(int(steps)):
        g.replay()
    cur.synchronize()
    for net in nets:
        net.steps += int(steps)
    out = [np.array([float(l)]) for l in losses]
    del g
    return out


def fourier_features(xy, n_freq=16, device="cuda", f_max=0.5, f_min=0.25):
    """(n, 2) coordinates in [-1, 1] -> (n, width) bf16 network inputs with
    ``n_freq`` frequencies geometrically spaced from f_min to f_max cycles per
    unit. Scan frames change smoothly with the motors: a low band keeps the
    network's interpolation between training frames smooth (measured on the
    4M-atom rocking scans: f_max = 0.5 generalises, a band reaching the
    training grid's Nyquist limit only aliases between training frames)."""
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


def _split_bf16(x):
    """x = hi + lo with both halves bf16 (16 mantissa bits together)."""
    hi = x.to(torch.bfloat16)
    lo = (x - hi.float()).to(torch.bfloat16)
    return hi.contiguous(), lo.contiguous()


class FrameBasis:
    """Principal components of the training frames' normalised intensity
    X = I / max I: the mean frame and ``rank`` orthonormal rows V (rank, P).
    Built from the Gram matrix of the centred frames in FP64 on the device
    and its n x n eigendecomposition on the host (FP64: the components the
    surrogate needs reach 1e-9 of the top variance, below an FP32 Gram
    product's round-off)."""

    def __init__(self, X, rank):
        n = int(X.shape[0])
        self.mu = X.mean(0).contiguous()
        Xc = (X - self.mu).double()
        lam, U = np.linalg.eigh((Xc @ Xc.T).cpu().numpy())
        order = np.argsort(lam)[::-1][: min(int(rank), n)]
        # drop components at the FP64 Gram product's round-off level
        # (centring alone removes one dimension)
        order = order[lam[order] > 1e-12 * max(float(lam.max()), 1e-300)]
        lam = lam[order]
        U = U[:, order]
        dev = X.device
        self.V = (torch.tensor(U / np.sqrt(lam), dtype=torch.float64, device=dev).T @ Xc
                  ).float().contiguous()
        self.rank = len(order)
        # decoding operand: per pixel [V_hi | V_lo | V_hi] (bf16, k-contiguous,
        # zero-padded to a multiple of 8), paired with [c_hi | c_hi | c_lo]
        r, P = self.rank, int(self.V.shape[1])
        self.k3 = (3 * r + 7) // 8 * 8
        V_hi, V_lo = _split_bf16(self.V)
        self.VT3 = torch.zeros((P, self.k3), dtype=torch.bfloat16, device=dev)
        self.VT3[:, :r] = V_hi.T
        self.VT3[:, r: 2 * r] = V_lo.T
        self.VT3[:, 2 * r: 3 * r] = V_hi.T

    def coefficients(self, X):
        """(m, P) normalised frames -> (m, rank) coefficients (X - mean) V^T."""
        return (X - self.mu) @ self.V.T

    def decode(self, net, coef, out=None, row_scale=None, row_map=None, clamp=False):
        """Frames coef V + mean from (m, rank) coefficients, in one tcgen05
        GEMM (net's mk_gemm_tc) with hi/lo operand splitting: coef and V are
        each split into two bf16 halves and the three products that matter
        (hi.hi + hi.lo + lo.hi) run as one product of K = 3 rank, FP32
        accumulation (~1e-5 relative). The epilogue adds the mean, clamps at
        0 (``clamp``), multiplies row m by ``row_scale[m]`` and stores it at
        row ``row_map[m]`` of ``out`` (default: a new (m, P) array)."""
        m, P, r = int(coef.shape[0]), int(self.V.shape[1]), self.rank
        if out is None:
            out = torch.empty((m, P), dtype=torch.float32, device=coef.device)
        if m == 0:
            return out
        ch, cl = _split_bf16(coef.float())
        A = torch.zeros((m, self.k3), dtype=torch.bfloat16, device=coef.device)
        A[:, :r] = ch
        A[:, r: 2 * r] = ch
        A[:, 2 * r: 3 * r] = cl
        net._gemm(m, P, self.k3, A, self.k3, 1, self.VT3, 1, self.k3, out, P, self.mu,
                  GEMM_BIAS | (GEMM_RELU if clamp else 0), None, 0, row_scale=row_scale,
                  row_map=row_map)
        return out


def spline_matrix(n, nodes):
    """(n, len(nodes)) weights of the interpolating cubic spline (not-a-knot
    ends) through values at the grid positions ``nodes`` (increasing
    integers), evaluated at positions 0 .. n-1: row p applied to the node
    values gives the spline at p. Two nodes give the straight line, one a
    constant."""
    nodes = np.asarray(nodes, dtype=np.float64)
    k = len(nodes)
    if k == 1:
        return np.ones((n, 1))
    from scipy.interpolate import CubicSpline
    return CubicSpline(nodes, np.eye(k), bc_type="not-a-knot")(np.arange(n, dtype=np.float64))


class SurrogateScan:
    """Surrogate-assisted theta x chi scan (see the module docstring).

    Args:
        beam, sample, detector, stage: as for BatchedScan / scan_nD.
        theta, chi: offsets [rad] added to the stage's mu and chi motors.
        roi: square ROI side (pixels) around the detector centre.
        stride: training frames every ``stride`` points along each axis (a
            grid of nodes; the last point of an axis is extrapolated to when
            ``stride`` does not divide its length minus one).
        judge_every, tol: exact re-judging cadence and fallback threshold.
        rank: principal components of the normalised frames (at most; the
            training frames' span and the FP64 round-off may give fewer).
        hidden, n_hidden, n_freq, f_max, f_min, fit_steps, lr, seed: the
            network (Fourier features of the two motor coordinates, ReLU
            layers) and its training.
        batch_frames: most frames per batched exact launch.
    """

    def __init__(self, beam, sample, detector, stage, theta, chi, roi=128, stride=4,
                 judge_every=8, tol=0.02, hidden=256, n_hidden=4, n_freq=16, fit_steps=2000,
                 lr=3e-3, seed=0, sc_kwargs=None, device="cuda", rank=64, f_max=0.5, f_min=0.25,
                 batch_frames=2048):
        self.beam, self.sample, self.detector, self.stage = beam, sample, detector, stage
        self.theta = np.asarray(theta, dtype=np.float64)
        self.chi = np.asarray(chi, dtype=np.float64)
        self.roi, self.stride = int(roi), int(stride)
        if self.stride < 1:
            raise ValueError("stride must be >= 1")
        self.judge_every, self.tol = int(judge_every), float(tol)
        self.hidden, self.n_hidden, self.n_freq = hidden, n_hidden, n_freq
        self.fit_steps, self.lr, self.seed = fit_steps, lr, seed
        self.rank, self.f_max, self.f_min = int(rank), float(f_max), float(f_min)
        self.batch_frames = int(batch_frames)
        self.kw = dict(apply_polarization=False, spherical_decay=False, remove_forward=False)
        self.kw.update(sc_kwargs or {})
        self.dev = torch.device(device)
        nt, nc = len(self.theta), len(self.chi)
        ii, jj = np.meshgrid(np.arange(nt), np.arange(nc), indexing="ij")
        self.ij = np.stack([ii.ravel(), jj.ravel()], 1)          # raster order
        norm = lambda v, n: (2.0 * v / max(n - 1, 1)) - 1.0
        self.xy = np.stack([norm(self.ij[:, 0], nt), norm(self.ij[:, 1], nc)], 1)
        self.nodes_t = np.arange(0, nt, self.stride)
        self.nodes_c = np.arange(0, nc, self.stride)
        self.train = (self.ij[:, 0] % self.stride == 0) & (self.ij[:, 1] % self.stride == 0)
        mu0 = float(stage.motor_value[stage.motor_index("mu")])
        chi0 = float(stage.motor_value[stage.motor_index("chi")])
        self.steps = [dict(mu=mu0 + self.theta[i], chi=chi0 + self.chi[j]) for i, j in self.ij]
        self._staged = None
        self._side, self._keep = None, []

    def prepare(self):
        """Stage the atoms and tiles once (setup shared by every exact call,
        and by an exact-only scan alike), and make the first call of every
        kernel and library routine the surrogate uses (module loading,
        library handles) on a throw-away problem of the scan's shapes, so
        that none of it lands in the timed phases."""
        if self._staged is not None:
            return
        self.exact(np.zeros(1, np.int64))
        n_nodes, P = len(self.nodes_t) * len(self.nodes_c), self.roi * self.roi
        n_tr = max(n_nodes, 2)
        I = torch.rand((n_tr, P), dtype=torch.float32, device=self.dev) + 0.5
        basis = FrameBasis(I / I.amax(1, keepdim=True), min(self.rank, n_tr - 1))
        T = self._targets(I, basis)
        base = self._spline_base(T[:n_nodes])
        sc = (T - base[: T.shape[0]]).std(0).clamp_min(1e-12)
        feats = fourier_features(self.xy[:n_tr], self.n_freq, self.dev, f_max=self.f_max,
                                 f_min=self.f_min)
        net = MLP(feats.shape[1], basis.rank + 1, hidden=32, n_hidden=2, seed=self.seed,
                  device=self.dev)
        Tf = ((T - base[: T.shape[0]]) / sc).float().contiguous()
        cw = (sc * sc / (sc * sc).sum() * sc.numel()).float().contiguous()
        net.fit(feats, Tf, steps=2, col_w=cw)
        net.fit_graph(feats, Tf, steps=2, col_w=cw)
        pair = MLP(feats.shape[1], basis.rank + 1, hidden=32, n_hidden=2, seed=self.seed,
                   device=self.dev, groups=2)
        pair.fit_graph(torch.stack([feats, feats]).contiguous(), torch.stack([Tf, Tf]).contiguous(),
                       steps=2, col_w=cw)
        pair.predict(feats)
        Y = 0.5 * (net.predict(feats) + net.predict(feats))
        I_pred = self._decode(net, basis, base[: T.shape[0]] + Y.double() * sc)
        err = frame_rel_error(I_pred[:4], I[:4])
        idx = torch.as_tensor([0, 1], device=self.dev)
        I_pred[idx] = I[:2]
        frames = torch.empty((n_tr, P), dtype=torch.float32, device=self.dev)
        frames[idx] = I_pred[:2]
        self._decode(net, basis, base[:2], out=frames, rows=idx)
        float(err.max())
        del I, I_pred, frames
        torch.cuda.synchronize()

    def _train_distance(self, idx):
        """Grid distance of each frame (indices into the scan) to its nearest
        training frame."""
        tr = self.ij[self.train].astype(np.float64)
        q = self.ij[np.asarray(idx)].astype(np.float64)
        d = np.full(len(q), np.inf)
        for c in range(0, len(tr), 512):
            t = tr[c: c + 512]
            d = np.minimum(d, np.sqrt(((q[:, None, :] - t[None, :, :]) ** 2).sum(-1)).min(1))
        return d

    def _targets(self, I, basis):
        """(m, rank + 1) FP64 description of exact frames: the coefficients
        of their peak-normalised intensity and the log of their peak."""
        M = I.amax(1, keepdim=True).clamp_min(1e-300)
        C = basis.coefficients(I / M)
        return torch.cat([C.double(), torch.log(M.double())], 1)

    def _spline_base(self, T_nodes):
        """The interpolating bicubic spline (not-a-knot) of the node frames'
        description ``T_nodes`` (training frames in raster order, a grid of
        len(nodes_t) x len(nodes_c)), at every frame of the scan: (n, c)."""
        nt, nc = len(self.theta), len(self.chi)
        Wt = torch.tensor(spline_matrix(nt, self.nodes_t), dtype=torch.float64, device=self.dev)
        Wc = torch.tensor(spline_matrix(nc, self.nodes_c), dtype=torch.float64, device=self.dev)
        G = T_nodes.reshape(len(self.nodes_t), len(self.nodes_c), -1)
        return torch.einsum("ia,abc,jb->ijc", Wt, G, Wc).reshape(nt * nc, -1)

    def _decode(self, net, basis, D, out=None, rows=None):
        """Intensities from descriptions D (m, rank + 1): the decoded
        normalised frame, clamped at 0, times the peak exp(D[:, rank]);
        into a new (m, P) array, or into rows ``rows`` (device int64) of
        ``out``."""
        r = basis.rank
        scale = torch.exp(D[:, r]).float().contiguous()
        return basis.decode(net, D[:, :r].float().contiguous(), out=out, row_scale=scale,
                            row_map=rows, clamp=True)

    def exact(self, idx, first=256):
        """Exact intensities (len(idx), roi*roi) of the given frames, in
        batched launches of at most ``batch_frames`` frames (the first of at
        most ``first``). The batches' sums run on a side stream, so that the
        set-up of the next batch (frame geometry on the host, pixel arrays
        and bounds on the device) overlaps the previous batch's sum; the
        small first batch keeps the set-up that cannot overlap short. The
        current stream waits for the result."""
        idx = np.asarray(idx)
        P = self.roi * self.roi
        if idx.size == 0:
            return torch.zeros((0, P), dtype=torch.float32, device=self.dev)
        if self._side is None:
            self._side = torch.cuda.Stream(self.dev)
        side = self._side
        side.synchronize()                  # the previous call's batches are done:
        self._keep = []                     # their buffers may go
        cur = torch.cuda.current_stream(self.dev)
        out = torch.empty((idx.size, P), dtype=torch.float32, device=self.dev)
        cuts = [0, min(int(first), idx.size)]
        while cuts[-1] < idx.size:
            cuts.append(min(cuts[-1] + self.batch_frames, idx.size))
        for a, b in zip(cuts[:-1], cuts[1:]):
            sub = idx[a:b]
            frames = frames_from_motors(self.stage, self.detector, [self.steps[i] for i in sub],
                                        [self.roi] * len(sub))
            if len(frames) == 1:           # a one-frame batch still goes through the scan path
                frames = frames * 2
            # no tuning inside the timed scan: the cached launch shape or the default
            scan = BatchedScan(self.beam, self.sample, frames, staged=self._staged, tune=False,
                               **self.kw)
            self._staged = self._staged or scan
            side.wait_stream(cur)
            with torch.cuda.stream(side):
                f, _ = scan.run(side)
                out[a:b] = (f * f).sum(1).reshape(len(frames), -1)[: len(sub)].float()
                done = torch.cuda.Event()
                done.record(side)
            # a batch's buffers stay alive until the side stream is done with
            # them; two batches back it long is
            while len(self._keep) >= 2:
                self._keep[0][1].synchronize()
                self._keep.pop(0)
            self._keep.append((scan, done))
        cur.wait_stream(side)
        return out

    def run(self, verify=0, exact_all=False):
        """Run the scan. ``exact_all`` also computes every frame exactly (the
        exact-only scan, timed) and the true error of every predicted frame;
        otherwise the exact-only time is the exact launch's per-frame time
        times the frame count, and ``verify`` > 0 computes that many unjudged
        predicted frames exactly (untimed) to measure their true error."""
        sync = torch.cuda.synchronize
        n = len(self.ij)
        t = {}
        sync()
        t0 = time.perf_counter()
        self.prepare()
        sync()
        setup_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        tr = np.flatnonzero(self.train)
        if tr.size < 2:
            raise ValueError("the surrogate needs at least two training frames")
        pred_idx = np.flatnonzero(~self.train)
        # Judging: the predicted frames in raster order form blocks of
        # judge_every; each block's judged frame is the one farthest from the
        # training frames (the hardest to interpolate), so a passing judge
        # vouches for the easier frames around it. The choice depends on the
        # frames' positions alone, so the training frames and the judged
        # frames are computed exactly in one batched launch.
        blocks = [np.arange(b, min(b + self.judge_every, len(pred_idx)))
                  for b in range(0, len(pred_idx), self.judge_every)]
        far = self._train_distance(pred_idx)
        judged = np.array([blk[int(np.argmax(far[blk]))] for blk in blocks], dtype=np.int64)
        fold = np.arange(len(judged)) % 2          # alternate blocks: two interleaved folds
        I_ex = self.exact(np.concatenate([tr, pred_idx[judged]]))
        I_train, I_j = I_ex[: tr.size], I_ex[tr.size:]
        sync()
        t["exact"] = time.perf_counter() - t0
        # The interpolating bicubic spline of the training frames' description
        # (principal-component coefficients and log peak) over the node grid
        # is the base; two networks learn its residual, each from the
        # training frames (residual 0) and the judged frames of one fold.
        t0 = time.perf_counter()
        M_tr = I_train.amax(1, keepdim=True).clamp_min(1e-300)
        basis = FrameBasis(I_train / M_tr, self.rank)
        r = basis.rank
        T_tr, T_j = self._targets(I_train, basis), self._targets(I_j, basis)
        base = self._spline_base(T_tr)
        R_tr = T_tr - base[torch.as_tensor(tr, device=self.dev)]
        R_j = T_j - base[torch.as_tensor(pred_idx[judged], device=self.dev)]
        scale = (R_j.std(0) if len(judged) > 1 else R_j.abs().amax(0)).clamp_min(1e-12)
        # network outputs padded to a multiple of 8 (16-byte rows for the
        # GEMMs); the padding columns carry zero targets and zero loss weight
        n_out = (r + 1 + 7) // 8 * 8
        col_w = torch.zeros(n_out, dtype=torch.float32, device=self.dev)
        col_w[: r + 1] = (scale * scale / (scale * scale).sum() * (r + 1)).float()
        feats = fourier_features(self.xy, self.n_freq, self.dev, f_max=self.f_max, f_min=self.f_min)
        # the two networks as one group of 2 (each GEMM launch serves both);
        # the shorter fold repeats its last row to give both the same batch
        Xs, Ts = [], []
        for f in (0, 1):
            rows = np.concatenate([tr, pred_idx[judged[fold == f]]])
            Tf = (torch.cat([R_tr, R_j[torch.as_tensor(fold == f, device=self.dev)]]) / scale).float()
            Ts.append(torch.nn.functional.pad(Tf, (0, n_out - (r + 1))))
            Xs.append(feats[torch.as_tensor(rows, device=self.dev)])
        nb = max(int(x.shape[0]) for x in Xs)
        grow = lambda x: torch.cat([x, x[-1:].expand(nb - x.shape[0], -1)]) if x.shape[0] < nb else x
        X2 = torch.stack([grow(x) for x in Xs]).contiguous()
        T2 = torch.stack([grow(x) for x in Ts]).contiguous()
        self.net = MLP(feats.shape[1], n_out, self.hidden, self.n_hidden, self.seed, self.dev, groups=2)
        self.losses = [self.net.fit_graph(X2, T2, steps=self.fit_steps, lr=self.lr, col_w=col_w)]
        sync()
        t["fit"] = time.perf_counter() - t0
        # Every judged frame is predicted by the network that did not train on
        # it; the other frames by the mean of the two.
        t0 = time.perf_counter()
        F = feats[torch.as_tensor(pred_idx, device=self.dev)]
        Y = self.net.predict(F)
        Y0, Y1 = Y[0, :, : r + 1], Y[1, :, : r + 1]
        corr = 0.5 * (Y0 + Y1)
        j0 = torch.as_tensor(judged[fold == 0], device=self.dev)
        j1 = torch.as_tensor(judged[fold == 1], device=self.dev)
        corr[j0] = Y1[j0]
        corr[j1] = Y0[j1]
        D = base[torch.as_tensor(pred_idx, device=self.dev)] + corr.double() * scale
        jd = torch.as_tensor(judged, device=self.dev)
        err_j = frame_rel_error(self._decode(self.net, basis, D[jd]), I_j).cpu().numpy()
        sync()
        t["predict_judge"] = time.perf_counter() - t0
        failed = [blk[blk != j] for blk, j, e in zip(blocks, judged, err_j) if e > self.tol]
        fb = np.concatenate(failed).astype(np.int64) if failed else np.zeros(0, np.int64)
        # The returned frames: training and judged frames exact, the failed
        # blocks' other frames exact, every other frame decoded straight into
        # its row of the output.
        t0 = time.perf_counter()
        frames = torch.empty((n, self.roi * self.roi), dtype=torch.float32, device=self.dev)
        frames[torch.as_tensor(tr, device=self.dev)] = I_train
        frames[torch.as_tensor(pred_idx[judged], device=self.dev)] = I_j
        keep = np.setdiff1d(np.arange(len(pred_idx)), np.concatenate([judged, fb]))
        self._decode(self.net, basis, D[torch.as_tensor(keep, device=self.dev)], out=frames,
                     rows=torch.as_tensor(pred_idx[keep], device=self.dev))
        sync()
        t["decode"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        if fb.size:
            frames[torch.as_tensor(pred_idx[fb], device=self.dev)] = self.exact(pred_idx[fb])
        sync()
        t["fallback"] = time.perf_counter() - t0
        total = sum(t.values())
        # the network's gain, held out: the judged frames from the spline alone
        I_base_j = self._decode(self.net, basis, base[torch.as_tensor(pred_idx[judged],
                                                                          device=self.dev)])
        err_jb = frame_rel_error(I_base_j, I_j).cpu().numpy()
        exact_frames = len(tr) + len(judged) + int(fb.size)
        res = dict(frames=frames, n_frames=n, n_train=len(tr), n_judged=len(judged),
                   n_fallback=int(fb.size), n_failed_judges=len(failed), exact_frames=exact_frames,
                   judge_err=err_j, judge_err_base=err_jb, times=t, setup_seconds=setup_s,
                   seconds=total, frames_per_s=n / total,
                   final_loss=float(self.losses[-1][-1]), params=self.net.n_params, rank=r)
        if exact_all:
            sync()
            t0 = time.perf_counter()
            I_all = self.exact(np.arange(n))
            sync()
            ex_s = time.perf_counter() - t0
            res.update(exact_seconds=ex_s, exact_measured=True)
            pi = torch.as_tensor(pred_idx, device=self.dev)
            # the prediction of every predicted frame (judged ones by the
            # network that did not see them), and the spline's alone
            I_b = self._decode(self.net, basis, D)
            res["model_err"] = frame_rel_error(I_b, I_all[pi]).cpu().numpy()
            self._decode(self.net, basis, base[pi], out=I_b)
            res["base_err"] = frame_rel_error(I_b, I_all[pi]).cpu().numpy()
            del I_b
            res["final_err"] = frame_rel_error(frames, I_all).cpu().numpy()
        else:
            res.update(exact_seconds=n * t["exact"] / (len(tr) + len(judged)), exact_measured=False)
        res["exact_frames_per_s"] = n / res["exact_seconds"]
        res["gain"] = res["exact_seconds"] / total
        sync()
        self._keep = []
        if verify and not exact_all:
            rng = np.random.default_rng(self.seed + 1)
            unjudged = np.setdiff1d(np.arange(len(pred_idx)), np.concatenate([judged, fb]))
            pick = rng.choice(unjudged, size=min(int(verify), unjudged.size), replace=False) \
                if unjudged.size else np.zeros(0, np.int64)
            I_true = self.exact(pred_idx[pick])
            res["verify_err"] = frame_rel_error(
                frames[torch.as_tensor(pred_idx[pick], device=self.dev)], I_true).cpu().numpy()
        return res
