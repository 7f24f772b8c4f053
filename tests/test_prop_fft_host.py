"""The fused spectral column pass (mk_prop_cols, mk_prop.cu) replayed on
the CPU: its in-place FFT -- bit-reversed load, radix-2
decimation-in-time stages fused three at a time (then two or one), each
butterfly reading and writing the same points -- for every power-of-two
length it takes, forward and inverse, against numpy's FFT, with every
shared-memory index inside the line and every point owned by exactly one
butterfly per pass. The GPU tests check the kernel itself against the
unfused propagation and the reference's own output."""
import numpy as np
import pytest


def bitrev(i, bits):
    return int(format(i, f"0{bits}b")[::-1], 2) if bits else 0


def groups(logn):
    out, left = [], logn
    while left >= 3:
        out.append(3)
        left -= 3
    if left:
        out.append(left)
    return out


def dit_fft(x, inv=False):
    """The kernel's transform of one line: load bit-reversed, then the fused
    in-place stage groups (mk_dit_pass), natural order out."""
    N = len(x)
    logn = int(np.log2(N))
    tw = np.exp(-2j * np.pi * np.arange(N) / N).astype(np.complex64)
    s = np.empty(N, np.complex64)
    for r in range(N):
        s[bitrev(r, logn)] = x[r]
    m = 1
    for G in groups(logn):
        R = 1 << G
        nb = N // R
        owned = np.zeros(N, int)
        for q in range(nb):
            i = q & (m - 1)
            base = (q - i) * R + i
            idx = [base + r * m for r in range(R)]
            assert min(idx) >= 0 and max(idx) < N
            owned[idx] += 1
            v = s[idx].astype(np.complex128)
            for h in range(G):
                hs = m << h
                tstep = N // (2 * hs)
                for a in range(R):
                    if a & (1 << h):
                        continue
                    j = i + (a & ((1 << h) - 1)) * m
                    assert j * tstep < N
                    w = tw[j * tstep]
                    if inv:
                        w = np.conj(w)
                    xa, y = v[a], v[a + (1 << h)] * w
                    v[a], v[a + (1 << h)] = xa + y, xa - y
            s[idx] = v
        assert (owned == 1).all()                      # every point in one butterfly
        m <<= G
    return s


@pytest.mark.parametrize("logn", range(1, 14))
def test_dit_passes_match_numpy(logn):
    N = 1 << logn
    rng = np.random.default_rng(logn)
    x = (rng.standard_normal(N) + 1j * rng.standard_normal(N)).astype(np.complex64)
    f = dit_fft(x)
    ref = np.fft.fft(x.astype(np.complex128))
    assert np.abs(f - ref).max() <= 5e-6 * np.abs(ref).max() * max(1, logn)
    b = dit_fft(f, inv=True)                             # natural-order input, as after H
    assert np.abs(b / N - x).max() <= 5e-6 * np.abs(x).max() * max(1, logn)


def test_stage_groups():
    assert groups(13) == [3, 3, 3, 3, 1]
    assert groups(12) == [3, 3, 3, 3]
    assert groups(2) == [2]
    assert groups(1) == [1]
    assert sum(groups(11)) == 11


def test_column_groups_and_shared_memory_indices():
    """mk_prop_cols_width and the load/store index maps: W columns of N
    points at stride N + 1 stay inside W (N + 1) points, each loaded once."""
    for ny2 in (2, 16, 1024, 8192):
        for logn in range(1, 14):
            N = 1 << logn
            W = max(1, min(16384 // N, 16, ny2))
            assert W * N <= 16384 and ny2 % W == 0
            ld = N + 1
            e = np.arange(W * N)
            r, c = e // W, e % W
            dst = c * ld + np.array([bitrev(int(v), logn) for v in r])
            assert dst.max() < W * ld and len(np.unique(dst)) == W * N
