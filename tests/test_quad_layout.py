"""The pixel-quad layout, checked on the CPU: the index arithmetic of the
quad kernels (mk_split.cuh, the PM == 2 pixel mapping and its store mask)
and the plan's block count (mk_scan_plan's quad slots), replayed in NumPy.
Every pixel of every frame shape must be stored exactly once, every load
must stay inside the frame, and the blocks the plan allots must reach every
quad."""
import numpy as np
import pytest


def plan_blocks(n_pix, row, nt, ppt):
    """mk_scan_plan: pixel slots of a quad frame and its pixel blocks."""
    rows = n_pix // row
    slots = 4 * ((row + 1) // 2) * ((rows + 1) // 2)
    return (slots + nt * ppt - 1) // (nt * ppt)


def kernel_pixels(n_pix, row, nt, ppt, pix_blocks):
    """(loads, stores) of all threads of all pixel blocks: the kernel's quad
    mapping, out-of-range quads set to n_pix (loads clamp, stores skip)."""
    nq = ppt // 4
    rows = n_pix // max(row, 1)
    half = (row + 1) >> 1
    n_quads = half * ((rows + 1) >> 1)
    loads, stores = [], []
    for pb in range(pix_blocks):
        for tid in range(nt):
            for j in range(nq):
                qi = pb * (nt * nq) + j * nt + tid
                if qi >= n_quads:
                    loads += [n_pix - 1] * 4
                    continue
                qz, qy = divmod(qi, half)
                r0, c0 = 2 * qz, 2 * qy
                r1, c1 = min(r0 + 1, rows - 1), min(c0 + 1, row - 1)
                pix = [r0 * row + c0, r0 * row + c1, r1 * row + c0, r1 * row + c1]
                keep = [True, c1 != c0, r1 != r0, c1 != c0 and r1 != r0]
                loads += pix
                stores += [p for p, k in zip(pix, keep) if k]
    return np.array(loads), np.array(stores)


SHAPES = [(1, 1), (1, 7), (7, 1), (2, 2), (3, 3), (15, 12), (16, 16), (13, 11), (24, 21),
          (64, 64), (33, 9), (128, 128), (487, 3)]


@pytest.mark.parametrize("nt,ppt", [(64, 4), (64, 8), (128, 4), (128, 8), (256, 4), (256, 8)])
def test_every_pixel_stored_once(nt, ppt):
    for ny, nz in SHAPES:
        n_pix = ny * nz
        pb = plan_blocks(n_pix, ny, nt, ppt)
        loads, stores = kernel_pixels(n_pix, ny, nt, ppt, pb)
        assert loads.min() >= 0 and loads.max() < n_pix, (ny, nz)
        assert len(stores) == n_pix, (ny, nz, len(stores))
        assert np.array_equal(np.sort(stores), np.arange(n_pix)), (ny, nz)


def test_quads_are_neighbours():
    """The four pixels of a quad are a 2x2 block of the detector (row-major,
    row length ny), or its repeated edge."""
    ny, nz = 13, 11
    loads, _ = kernel_pixels(ny * nz, ny, 64, 4, plan_blocks(ny * nz, ny, 64, 4))
    for a, b, c, d in loads.reshape(-1, 4)[: ((ny + 1) // 2) * ((nz + 1) // 2)]:
        ra, ca = divmod(a, ny)
        assert divmod(b, ny) in ((ra, ca + 1), (ra, ca))
        assert divmod(c, ny) in ((ra + 1, ca), (ra, ca))
        rd, cd = divmod(d, ny)
        assert (rd - ra, cd - ca) in ((1, 1), (0, 1), (1, 0), (0, 0))


def octet_pixels(n_pix, row, nt, pix_blocks):
    """(loads, stores) of the octet kernels' mapping (mk_split.cuh, PM == 3):
    thread gi = pb * nt + tid owns rows 2 gz, 2 gz + 1 and columns
    4 gy .. 4 gy + 3 (pixels 0..3 the left quad a b c d, 4..7 the right one);
    past the last octet the pixels are n_pix (loads clamp, stores skip)."""
    rows = n_pix // row
    gpr = row >> 2
    n_oct = gpr * (rows >> 1)
    loads, stores = [], []
    for pb in range(pix_blocks):
        for tid in range(nt):
            gi = pb * nt + tid
            if gi >= n_oct:
                loads += [n_pix - 1] * 8
                continue
            gz, gy = divmod(gi, gpr)
            a0 = 2 * gz * row + 4 * gy
            c0 = a0 + row
            pix = []
            for j in range(2):
                pix += [a0 + 2 * j, a0 + 2 * j + 1, c0 + 2 * j, c0 + 2 * j + 1]
            loads += pix
            stores += pix
    return np.array(loads), np.array(stores)


OCTET_SHAPES = [(4, 2), (8, 2), (4, 6), (16, 16), (64, 64), (128, 128), (20, 14), (512, 2), (4, 512)]


@pytest.mark.parametrize("nt", [64, 128, 256])
def test_octets_store_every_pixel_once(nt):
    for ny, nz in OCTET_SHAPES:
        n_pix = ny * nz
        pb = (n_pix + nt * 8 - 1) // (nt * 8)      # mk_scan_plan: whole octets, 8 pixels a thread
        loads, stores = octet_pixels(n_pix, ny, nt, pb)
        assert loads.min() >= 0 and loads.max() < n_pix, (ny, nz)
        assert len(stores) == n_pix and np.array_equal(np.sort(stores), np.arange(n_pix)), (ny, nz)


def test_octets_are_two_side_by_side_quads():
    ny, nz = 20, 6
    loads, _ = octet_pixels(ny * nz, ny, 64, 1)
    for o in loads.reshape(-1, 8)[: (ny // 4) * (nz // 2)]:
        r, c = divmod(int(o[0]), ny)
        assert r % 2 == 0 and c % 4 == 0
        want = [(r, c), (r, c + 1), (r + 1, c), (r + 1, c + 1),
                (r, c + 2), (r, c + 3), (r + 1, c + 2), (r + 1, c + 3)]
        assert [divmod(int(p), ny) for p in o] == want


def square_pixels(n_pix, row, nt, pix_blocks):
    """(loads, stores) of the square kernels' mapping (mk_split.cuh, PM == 4):
    thread gi = pb * nt + tid owns rows 4 gz .. 4 gz + 3 and columns
    4 gy .. 4 gy + 3, pixels 4j..4j+3 the quad a b c d at rows 4 gz + 2 (j >> 1)
    (+1) and columns 4 gy + 2 (j & 1) (+1); past the last square the pixels
    are n_pix (loads clamp, stores skip)."""
    rows = n_pix // row
    gpr = row >> 2
    n_sq = gpr * (rows >> 2)
    loads, stores = [], []
    for pb in range(pix_blocks):
        for tid in range(nt):
            gi = pb * nt + tid
            if gi >= n_sq:
                loads += [n_pix - 1] * 16
                continue
            gz, gy = divmod(gi, gpr)
            base = 4 * gz * row + 4 * gy
            pix = []
            for j in range(4):
                a0 = base + 2 * (j >> 1) * row + 2 * (j & 1)
                pix += [a0, a0 + 1, a0 + row, a0 + row + 1]
            loads += pix
            stores += pix
    return np.array(loads), np.array(stores)


SQUARE_SHAPES = [(4, 4), (8, 4), (4, 8), (16, 16), (64, 64), (128, 128), (20, 12), (512, 4),
                 (4, 512), (256, 256)]


def test_squares_store_every_pixel_once():
    nt = 128
    for ny, nz in SQUARE_SHAPES:
        n_pix = ny * nz
        pb = (n_pix + nt * 16 - 1) // (nt * 16)    # mk_scan_plan: whole squares, 16 pixels a thread
        loads, stores = square_pixels(n_pix, ny, nt, pb)
        assert loads.min() >= 0 and loads.max() < n_pix, (ny, nz)
        assert len(stores) == n_pix and np.array_equal(np.sort(stores), np.arange(n_pix)), (ny, nz)


def test_squares_are_four_quads_in_a_square():
    """Quad j sits at row pair j >> 1 and column pair j & 1 of its square,
    which is the order the kernel's quad phases assume (columns s = -1 for
    quads 0, 2; rows t = -1 for quads 0, 1)."""
    ny, nz = 20, 12
    loads, _ = square_pixels(ny * nz, ny, 64, 1)
    for sq in loads.reshape(-1, 16)[: (ny // 4) * (nz // 4)]:
        r, c = divmod(int(sq[0]), ny)
        assert r % 4 == 0 and c % 4 == 0
        want = []
        for j in range(4):
            rr, cc = r + 2 * (j >> 1), c + 2 * (j & 1)
            want += [(rr, cc), (rr, cc + 1), (rr + 1, cc), (rr + 1, cc + 1)]
        assert [divmod(int(p), ny) for p in sq] == want
