"""The algebra of the octet (2x4) and square (4x4) pixel forms, checked on
the CPU in FP64: the device loops' formulas (mk_tile_terms_oct,
mk_tile_terms_sq, mk_octet_tile, mk_square_tile in csrc/mk_split.cuh) --
the group's mean phase, the shared half differences u and v, the quad
phases sigma_c +- 2u (+- 2v), the four sums K, R, S, Q of each quad and the
reconstruction A(s, t) = K - s t Q + i t R + i s S -- replayed in NumPy
with exact cos/sin for the half differences, against the direct sum
sum_a E_a exp(2 pi i D_a . w_p) of every pixel. The two agree to the phase
the form drops (the departure of w from the kernel's plane, times 2 pi |D|),
which is what the host bounds; with w exactly planar they agree to round-off.
"""
import numpy as np
import pytest


def _group_w(rows, cols, rng, curvature):
    """w of a rows x cols pixel group (row-major), a plane plus a small
    quadratic term of the pixel offsets."""
    g = rng.standard_normal(3) * 0.02        # row step of w (cycles per cycle of D)
    h = rng.standard_normal(3) * 0.02        # column step
    c = rng.standard_normal(3)
    q = rng.standard_normal((3, 3)) * curvature
    w = np.empty((rows, cols, 3))
    for r in range(rows):
        for k in range(cols):
            m, t = k - (cols - 1) / 2, r - (rows - 1) / 2
            w[r, k] = c + m * g + t * h + q[0] * m * m + q[1] * t * t + q[2] * m * t
    return w


def _quads(w):
    """The group's quads in the kernel's order, each (a, b, c, d) = rows
    r, r + 1 by columns k, k + 1: pixel index 4j + e."""
    rows, cols = w.shape[:2]
    out = []
    for r in range(0, rows, 2):
        for k in range(0, cols, 2):
            out.append(np.stack([w[r, k], w[r, k + 1], w[r + 1, k], w[r + 1, k + 1]]))
    return out


def _form_sum(w, D, E):
    """The octet / square form: one phase per quad from the group's mean,
    shared half differences, K R S Q sums, reconstruction."""
    rows, cols = w.shape[:2]
    quads = _quads(w)
    nq = len(quads)
    s_c = w.reshape(-1, 3).mean(0)
    hp = 0.5 * np.pi / nq
    u_vec = hp * sum((q[1] - q[0]) + (q[3] - q[2]) for q in quads)
    v_vec = hp * sum((q[2] - q[0]) + (q[3] - q[1]) for q in quads)
    sig = 2 * np.pi * D @ s_c                         # radians
    du, dv = D @ u_vec, D @ v_vec
    # quad centres: column pair offsets -1, +1 (octets, squares), row pair
    # offsets -1, +1 (squares); a pixel step is 2u along a row, 2v across
    centres = []
    for r in range(0, rows, 2):
        for k in range(0, cols, 2):
            sc = (k + 1 - (cols - 1) / 2) - 0.5      # -1 or +1 (units of a quad step)
            tc = (r + 1 - (rows - 1) / 2) - 0.5 if rows > 2 else 0.0
            centres.append((np.sign(sc) if cols > 2 else 0.0, np.sign(tc) if rows > 2 else 0.0))
    cu, su, cv, sv = np.cos(du), np.sin(du), np.cos(dv), np.sin(dv)
    pcc, pcs, psc, pss = cu * cv, cu * sv, su * cv, su * sv
    A = np.zeros((rows, cols), dtype=complex)
    for j, (qs, qt) in enumerate(centres):
        ph = sig + qs * 2 * du + qt * 2 * dv
        e = E * np.exp(1j * ph)
        K, R, S, Q = (e * pcc).sum(), (e * pcs).sum(), (e * psc).sum(), (e * pss).sum()
        a = K - Q + 1j * (-R) + 1j * (-S)            # (s, t) = (-, -)
        b = K + Q + 1j * (-R) + 1j * S                # (+, -)
        c = K + Q + 1j * R + 1j * (-S)                # (-, +)
        d = K - Q + 1j * R + 1j * S                   # (+, +)
        r0 = 2 * (j // (cols // 2))
        k0 = 2 * (j % (cols // 2))
        A[r0, k0], A[r0, k0 + 1], A[r0 + 1, k0], A[r0 + 1, k0 + 1] = a, b, c, d
    return A


def _direct_sum(w, D, E):
    return np.einsum("a,rka->rk", E, np.exp(2j * np.pi * np.einsum("ai,rki->rka", D, w)))


def _plane_residual(w):
    """Largest |w_p - plane_p| for the kernel's plane (mean plus offsets
    times the means of the within-quad steps)."""
    rows, cols = w.shape[:2]
    quads = _quads(w)
    nq = len(quads)
    g = sum((q[1] - q[0]) + (q[3] - q[2]) for q in quads) / (2 * nq)
    h = sum((q[2] - q[0]) + (q[3] - q[1]) for q in quads) / (2 * nq)
    mean = w.reshape(-1, 3).mean(0)
    worst = 0.0
    for r in range(rows):
        for k in range(cols):
            model = mean + (k - (cols - 1) / 2) * g + (r - (rows - 1) / 2) * h
            worst = max(worst, float(np.linalg.norm(w[r, k] - model)))
    return worst


@pytest.mark.parametrize("shape", [(2, 4), (4, 4)])
def test_planar_w_is_exact(shape):
    """With w exactly planar over the group the form drops nothing: its
    result equals the direct sum to round-off."""
    rng = np.random.default_rng(1)
    w = _group_w(*shape, rng, curvature=0.0)
    D = rng.uniform(-20, 20, (300, 3))                # cycles
    E = rng.uniform(0.5, 2.0, 300) * np.exp(1j * rng.uniform(-np.pi, np.pi, 300))
    A = _form_sum(w, D, E)
    ref = _direct_sum(w, D, E)
    assert np.abs(A - ref).max() <= 1e-9 * np.abs(E).sum()


@pytest.mark.parametrize("shape", [(2, 4), (4, 4)])
def test_curved_w_within_the_dropped_phase(shape):
    """With a curved w the difference stays within the dropped phase the
    host bounds: 2 pi max|D| x the plane residual, times sum |E|."""
    rng = np.random.default_rng(2)
    w = _group_w(*shape, rng, curvature=2e-6)
    D = rng.uniform(-20, 20, (300, 3))
    E = rng.uniform(0.5, 2.0, 300) * np.exp(1j * rng.uniform(-np.pi, np.pi, 300))
    A = _form_sum(w, D, E)
    ref = _direct_sum(w, D, E)
    dropped = 2 * np.pi * np.linalg.norm(D, axis=1).max() * _plane_residual(w)
    err = np.abs(A - ref).max()
    assert 0.0 < err <= dropped * np.abs(E).sum()
    assert dropped < 1e-2                              # the check is not vacuous
