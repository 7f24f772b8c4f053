"""The fused spectral row pass (mk_prop_rows, mk_prop.cu) replayed on the
CPU: its Stockham pass sequence (radix 8, then 4 or 2; the same read,
twiddle and write indices) against numpy's FFT for every power-of-two row
length it takes, and every shared-memory index inside the row. The GPU test
checks the kernel itself against the unfused propagation and the
reference's own output."""
import numpy as np
import pytest


def radices(logn):
    out, left = [], logn
    while left >= 3:
        out.append(8)
        left -= 3
    if left:
        out.append(1 << left)
    return out


def dft_small(v, R, inv):
    """The in-register R-point DFT (natural order), over the last axis."""
    n = np.arange(R)
    W = np.exp((2j if inv else -2j) * np.pi * np.outer(n, n) / R)
    return v @ W.T


def stockham(x, inv=False):
    N = x.shape[-1]
    logn = int(np.log2(N))
    tw = np.exp(-2j * np.pi * np.arange(N) / N).astype(np.complex64)
    src = x.astype(np.complex64).copy()
    Ns = 1
    for R in radices(logn):
        nb = N // R
        j = np.arange(nb)
        r = np.arange(R)
        idx_in = j[:, None] + r[None, :] * nb
        assert idx_in.min() >= 0 and idx_in.max() < N
        v = src[..., idx_in]                                  # (..., nb, R)
        k = j & (Ns - 1)
        tstep = N // (Ns * R)
        ti = (r[None, :] * k[:, None]) * tstep
        assert ti.max() < N
        w = tw[ti]
        if inv:
            w = np.conj(w)
        if Ns > 1:
            v = v * w
        v = dft_small(v, R, inv)
        base = (j - k) * R + k
        idx_out = base[:, None] + r[None, :] * Ns
        assert idx_out.min() >= 0 and idx_out.max() < N
        assert len(np.unique(idx_out)) == N                    # every point written once
        dst = np.empty_like(src)
        dst[..., idx_out] = v
        src = dst
        Ns *= R
    return src


@pytest.mark.parametrize("logn", range(1, 14))
def test_stockham_passes_match_numpy(logn):
    N = 1 << logn
    rng = np.random.default_rng(logn)
    x = (rng.standard_normal((3, N)) + 1j * rng.standard_normal((3, N))).astype(np.complex64)
    f = stockham(x)
    ref = np.fft.fft(x.astype(np.complex128), axis=-1)
    assert np.abs(f - ref).max() <= 5e-6 * np.abs(ref).max() * max(1, logn)
    b = stockham(f, inv=True)
    assert np.abs(b / N - x).max() <= 5e-6 * np.abs(x).max() * max(1, logn)


def test_radix_sequence():
    assert radices(13) == [8, 8, 8, 8, 2]
    assert radices(12) == [8, 8, 8, 8]
    assert radices(2) == [4]
    assert radices(1) == [2]
    assert np.prod(radices(11)) == 2048


def kernel_dft(v, inv):
    """mk_dft<R> as written in the kernel: DFT-4 by two radix-2 stages, DFT-8
    as DFT-4 of the even and odd points, the odd ones twiddled by
    exp(-/+ 2 pi i m / 8)."""
    R = len(v)
    if R == 2:
        return [v[0] + v[1], v[0] - v[1]]
    if R == 4:
        a0, a1 = v[0] + v[2], v[0] - v[2]
        b0, b1 = v[1] + v[3], (v[1] - v[3]) * (1j if inv else -1j)
        return [a0 + b0, a1 + b1, a0 - b0, a1 - b1]
    e, o = kernel_dft(v[0::2], inv), kernel_dft(v[1::2], inv)
    h = 0.70710678118654752
    sg = 1.0 if inv else -1.0
    o = [o[0], o[1] * (h + 1j * sg * h), o[2] * (1j if inv else -1j), o[3] * (-h + 1j * sg * h)]
    return [e[m] + o[m] for m in range(4)] + [e[m] - o[m] for m in range(4)]


@pytest.mark.parametrize("R", [2, 4, 8])
@pytest.mark.parametrize("inv", [False, True])
def test_in_register_dft_matches_the_definition(R, inv):
    rng = np.random.default_rng(R)
    v = rng.standard_normal(R) + 1j * rng.standard_normal(R)
    got = np.array(kernel_dft(list(v), inv))
    assert np.abs(got - dft_small(v, R, inv)).max() < 1e-12
