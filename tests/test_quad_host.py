"""Host logic of the pixel-sharing forms (no GPU): the quad differences of a
flat detector, the bounds that admit pairs and quads, and the clamping of a
launch shape to what the geometry and the kernels allow."""
import types

import numpy as np
import pytest
import torch

from mosaic_gb300 import engine


def _flat_pixels(ny, nz, pitch, dist, y0=0.0, z0=0.0, frames=None):
    """Stub with the attributes Pixels' bound methods read: a flat detector
    at x = dist, row index z, column index y (index iz * ny + iy)."""
    shapes = frames or [(ny, nz)]
    xyz, spans, off = [], [], 0
    for fny, fnz in shapes:
        y = y0 + pitch * (np.arange(fny) - 0.5 * (fny - 1))
        z = z0 + pitch * (np.arange(fnz) - 0.5 * (fnz - 1))
        Z, Y = np.meshgrid(z, y, indexing="ij")
        xyz.append(np.stack([np.full(Y.size, dist), Y.ravel(), Z.ravel()], 1))
        spans.append((off, fny * fnz))
        off += fny * fnz
    st = types.SimpleNamespace(xyz=torch.tensor(np.concatenate(xyz)), spans=spans, shapes=shapes)
    st.n = off
    st.quad_steps = lambda: engine.Pixels.quad_steps(st)
    st.octets_fit = lambda: engine.Pixels.octets_fit(st)
    st.octet_steps = lambda: engine.Pixels.octet_steps(st)
    st.squares_fit = lambda: engine.Pixels.squares_fit(st)
    st.square_steps = lambda: engine.Pixels.square_steps(st)
    u = st.xyz / torch.linalg.vector_norm(st.xyz, dim=1, keepdim=True)
    st.u = torch.cat([u.float(), torch.zeros(off, 1)], 1)
    st.pair_step = lambda: engine.Pixels.pair_step(st)
    st.r0_min = lambda: float(torch.linalg.vector_norm(st.xyz, dim=1).min())
    return st


def _tiles(radius, origin=0.0, radii=None):
    """Stub tiles: four of ``radius`` (or the given radii)."""
    radii = [radius] * 4 if radii is None else list(radii)
    org = torch.zeros((len(radii), 4), dtype=torch.float64)
    org[:, 3] = torch.tensor(radii, dtype=torch.float64)
    return types.SimpleNamespace(n_tiles=len(radii), max_radius=lambda: max(radii),
                                 max_origin_norm=lambda: origin, origin=org)


def test_quad_steps_of_a_flat_detector():
    p, R = 55e-6, 1.0
    pix = _flat_pixels(16, 12, p, R)
    st = pix.quad_steps()
    # row and cross-row differences: two pixel steps; mixed: second order
    assert st["row"] == pytest.approx(2 * p / R, rel=1e-3)
    assert st["col"] == pytest.approx(2 * p / R, rel=1e-3)
    assert st["diag"] == pytest.approx(np.sqrt(2) * p / R, rel=1e-3)
    assert st["mixed"] < 3 * (p / R) ** 2 * (16 * p / R)
    # off-centre the mixed difference grows like y z / R^2 (p/R)^2
    far = _flat_pixels(16, 12, p, R, y0=0.05, z0=0.04).quad_steps()
    assert st["mixed"] < far["mixed"] < 10 * (p / R) ** 2
    # odd sides: the kernel repeats the edge pixel, so the quads across it
    # have a zero difference there and the bounds are those of the rest
    odd = _flat_pixels(15, 11, p, R).quad_steps()
    even = _flat_pixels(14, 10, p, R).quad_steps()
    for key in ("row", "col", "diag"):
        assert odd[key] == pytest.approx(even[key], rel=2e-3), key
    assert odd["mixed"] < 3 * (p / R) ** 2 * (16 * p / R)
    one_col = _flat_pixels(1, 7, p, R).quad_steps()
    assert one_col["row"] == 0.0 and one_col["mixed"] == 0.0
    assert one_col["col"] == pytest.approx(2 * p / R, rel=1e-3)
    multi = _flat_pixels(0, 0, p, R, frames=[(8, 4), (15, 16), (7, 3), (8, 4)])
    ms = multi.quad_steps()
    assert ms["row"] == pytest.approx(2 * p / R, rel=2e-3)


def test_grouping_levels():
    k = 2 * np.pi / 1.2398e-10
    pix = _flat_pixels(16, 16, 55e-6, 1.0)
    tiles = _tiles(4.6e-8, 6e-8)
    level, info = engine.pixel_grouping(tiles, pix, k, 1e-6)
    assert level == 2
    assert info["quad_cross_rad"] < 1e-6
    # the quad half differences match the pair half difference
    assert info["quad_delta_rad"] == pytest.approx(info["pair_delta_rad"], rel=2e-2)
    # no budget left: pairs only; odd sides: quads still (the edge repeats),
    # but an odd row length puts a pair across each row end, so no pairs;
    # analyser: none
    assert engine.pixel_grouping(tiles, pix, k, 1e-12)[0] == 1
    assert engine.pixel_grouping(tiles, _flat_pixels(16, 15, 55e-6, 1.0), k, 1e-6)[0] == 2
    lv, inf = engine.pixel_grouping(tiles, _flat_pixels(15, 16, 55e-6, 1.0), k, 1e-6)
    assert lv == 2 and not inf["pairs_ok"]
    assert engine.pixel_grouping(tiles, _flat_pixels(15, 16, 55e-6, 1.0), k, 1e-12)[0] == 0
    lv, inf = engine.pixel_grouping(tiles, pix, k, 1e-6, analyser=1)     # top-hat: quads
    assert lv == 2 and not inf["pairs_ok"]
    lv, inf = engine.pixel_grouping(tiles, pix, k, 1e-6, analyser=2)     # Darwin: none
    assert lv == 0 and not inf["pairs_ok"]
    lv, inf = engine.pixel_grouping(tiles, pix, k, 1e-12, analyser=1)    # no budget: none
    assert lv == 0
    # pitch so coarse that the half difference passes 0.5 rad: none
    assert engine.pixel_grouping(tiles, _flat_pixels(16, 16, 2e-2, 1.0), k, 1e-6)[0] == 0
    # the |d|^2 term's change across the quad counts against the budget
    c0 = engine.quad_bounds(tiles, pix, k)["cross"]
    c1 = engine.quad_bounds(tiles, pix, k, fresnel_rad=1e-3)["cross"]
    assert c1 == pytest.approx(c0 + 2e-3 * pix.quad_steps()["diag"], rel=1e-9)


def test_grouping_launch_clamps_the_mode():
    k = 2 * np.pi / 1.2398e-10
    pix = _flat_pixels(16, 16, 55e-6, 1.0)
    tiles = _tiles(4.6e-8, 6e-8)
    level, info = engine.pixel_grouping(tiles, pix, k, 1e-6)
    cfg = engine.grouping_launch(dict(pix_per_thread=4, threads=128, pairs=2), level, tiles, pix, k,
                                 info)
    assert cfg["pairs"] == 2 and cfg["pair_short_radius_m"] == info["quad_short_radius_m"]
    cfg = engine.grouping_launch(dict(pix_per_thread=2, threads=128, pairs=2), level, tiles, pix, k,
                                 info)
    assert cfg["pairs"] == 1
    assert cfg["pair_short_radius_m"] == engine.pair_short_radius(tiles, pix, k)
    cfg = engine.grouping_launch(dict(pix_per_thread=1, threads=256, pairs=2), level, tiles, pix, k,
                                 info)
    assert cfg["pairs"] == 0 and cfg["pair_short_radius_m"] == 0.0
    cfg = engine.grouping_launch(dict(pix_per_thread=8, threads=64, pairs=2), 1, tiles, pix, k, info)
    assert cfg["pairs"] == 1
    cfg = engine.grouping_launch(dict(pix_per_thread=4, threads=128, pairs=1), 0, tiles, pix, k, info)
    assert cfg["pairs"] == 0
    # quads legal, pairs not (odd rows): a 2-pixel shape falls to one sin/cos a term
    odd = _flat_pixels(15, 16, 55e-6, 1.0)
    lv, inf = engine.pixel_grouping(tiles, odd, k, 1e-6)
    assert engine.grouping_launch(dict(pix_per_thread=8, threads=128, pairs=2), lv, tiles, odd, k,
                                  inf)["pairs"] == 2
    assert engine.grouping_launch(dict(pix_per_thread=2, threads=128, pairs=2), lv, tiles, odd, k,
                                  inf)["pairs"] == 0
    assert engine.grouping_launch(dict(pix_per_thread=4, threads=128, pairs=1), lv, tiles, odd, k,
                                  inf)["pairs"] == 0


def test_autotune_pick_keeps_the_default_within_noise():
    from mosaic_gb300 import autotune
    d = engine.default_launch(2)
    a = dict(pix_per_thread=8, threads=64, slices=0, pairs=2)
    b = dict(pix_per_thread=4, threads=128, slices=0, pairs=2)
    assert autotune.pick([a, d, b], [6.40, 6.43, 6.50], 2) == d      # 0.5 %: keep
    assert autotune.pick([a, d, b], [6.00, 6.43, 6.50], 2) == a      # 7 %: switch
    assert autotune.pick([a, b], [6.40, 6.30], 2) == b               # no default
    assert engine.default_launch(2)["pix_per_thread"] == 8
    assert engine.default_launch(1) == dict(pix_per_thread=4, threads=128, slices=0, pairs=1)


def test_analyser_launch_shapes():
    q = engine.analyser_launch(dict(pix_per_thread=8, threads=64, pairs=2))
    assert (q["threads"], q["pix_per_thread"], q["pairs"]) == (128, 8, 2)
    q = engine.analyser_launch(dict(pix_per_thread=4, threads=256, pairs=2))
    assert (q["threads"], q["pix_per_thread"]) == (256, 4)
    q = engine.analyser_launch(dict(pix_per_thread=8, threads=128, pairs=0))
    assert (q["threads"], q["pix_per_thread"]) in engine.ANALYSER_LAUNCHES


def test_octet_bounds_of_a_flat_detector():
    """The octet's departure from a plane is the row curvature of the pixel
    directions, ~(p/R)^2 / 2 near the axis; frames that are not whole
    octets have none; small tiles admit octets, large ones only quads."""
    k = 2 * np.pi / 1.2398e-10
    p, R = 55e-6, 1.0
    pix = _flat_pixels(16, 14, p, R)     # whole octets, not whole 4x4 squares
    st = pix.octet_steps()
    assert 0.3 * (p / R) ** 2 < st["plane"] < 1.0 * (p / R) ** 2
    assert st["step"] == pytest.approx(p / R, rel=1e-3)
    assert st["extent"] == pytest.approx(np.hypot(1.5, 0.5) * p / R, rel=1e-2)
    for shape in ((15, 16), (16, 15), (18, 16), (2, 2)):
        assert _flat_pixels(*shape, p, R).octet_steps() is None, shape
    multi = _flat_pixels(0, 0, p, R, frames=[(8, 4), (16, 14), (4, 2)])
    assert multi.octet_steps()["plane"] == pytest.approx(st["plane"], rel=0.5)
    assert _flat_pixels(0, 0, p, R, frames=[(8, 4), (6, 2)]).octet_steps() is None
    small, big = _tiles(2e-9, 6e-8), _tiles(4.6e-8, 6e-8)
    lv, info = engine.pixel_grouping(small, pix, k, 1e-6)
    assert lv == 3 and info["octet_cross_rad"] < 1e-6 and info["octet_tile_fraction"] == 1.0
    assert info["octet_cross_rad"] > info["quad_cross_rad"]
    assert small.max_radius() < info["octet_radius_m"] < big.max_radius()
    # every tile too wide: quads; a few wide tiles among narrow ones: octets
    # (the wide ones take the quad form inside the octet kernel)
    lv, info = engine.pixel_grouping(big, pix, k, 1e-6)
    assert lv == 2 and info["octet_tile_fraction"] == 0.0
    mixed = _tiles(0, 6e-8, radii=[2e-9] * 7 + [4.6e-8])
    lv, info = engine.pixel_grouping(mixed, pix, k, 1e-6)
    assert lv == 3 and info["octet_tile_fraction"] == pytest.approx(7 / 8)
    cfg = engine.grouping_launch(dict(pix_per_thread=8, threads=128, pairs=3), lv, mixed, pix, k,
                                 info)
    assert cfg["octet_radius_m"] == info["octet_radius_m"]
    assert engine.pixel_grouping(small, _flat_pixels(18, 16, p, R), k, 1e-6)[0] == 2
    assert engine.pixel_grouping(small, pix, k, 1e-6, analyser=1)[0] == 2
    # the radius shrinks linearly with the budget
    r1 = engine.octet_bounds(small, pix, k, 1e-6)["radius_m"]
    r2 = engine.octet_bounds(small, pix, k, 2e-6)["radius_m"]
    assert r2 == pytest.approx(2 * r1, rel=1e-9)
    # the |d|^2 term's change across the octet counts against the budget
    c0 = engine.octet_bounds(small, pix, k, 1e-6)["cross"]
    c1 = engine.octet_bounds(small, pix, k, 1e-6, fresnel_rad=1e-3)["cross"]
    assert c1 == pytest.approx(c0 + 4e-3 * st["extent"], rel=1e-9)
    assert engine.octet_bounds(small, pix, k, 1e-6, fresnel_rad=1.0)["radius_m"] == 0.0


def test_octet_launch_clamps():
    k = 2 * np.pi / 1.2398e-10
    pix = _flat_pixels(16, 14, 55e-6, 1.0)
    small = _tiles(2e-9, 6e-8)
    lv, info = engine.pixel_grouping(small, pix, k, 1e-6)
    assert lv == 3
    g = lambda cfg, level=lv: engine.grouping_launch(cfg, level, small, pix, k, info)
    cfg = g(dict(pix_per_thread=8, threads=128, pairs=3))
    assert cfg["pairs"] == 3 and cfg["pair_short_radius_m"] == info["quad_short_radius_m"]
    assert cfg["octet_radius_m"] == info["octet_radius_m"] > 0
    assert g(dict(pix_per_thread=8, threads=128, pairs=2))["octet_radius_m"] == 0.0
    assert g(dict(pix_per_thread=4, threads=128, pairs=3))["pairs"] == 2
    assert g(dict(pix_per_thread=8, threads=128, pairs=3), 2)["pairs"] == 2
    assert engine.default_launch(3) == dict(pix_per_thread=8, threads=128, slices=0, pairs=3)
    assert engine.analyser_launch(dict(pix_per_thread=8, threads=128, pairs=3))["pairs"] == 2


def test_square_bounds_of_a_flat_detector():
    """The square's departure from the kernel's plane (the mean plus the
    quads' mean row and column steps) is the curvature of the pixel
    directions along and across rows, ~(p/R)^2 near the axis; frames that
    are not whole squares have none; narrow tiles admit squares, wider ones
    octets (whose bound is smaller), the widest only quads."""
    k = 2 * np.pi / 1.2398e-10
    p, R = 55e-6, 1.0
    pix = _flat_pixels(16, 16, p, R)
    st = pix.square_steps()
    assert 0.3 * (p / R) ** 2 < st["plane"] < 2.0 * (p / R) ** 2
    assert st["plane"] > pix.octet_steps()["plane"]
    assert st["step"] == pytest.approx(p / R, rel=1e-3)
    assert st["extent"] == pytest.approx(np.hypot(1.5, 1.5) * p / R, rel=1e-2)
    for shape in ((16, 14), (14, 16), (16, 18), (2, 2), (4, 2)):
        assert _flat_pixels(*shape, p, R).square_steps() is None, shape
    multi = _flat_pixels(0, 0, p, R, frames=[(8, 4), (16, 16), (4, 8)])
    assert multi.square_steps()["plane"] == pytest.approx(st["plane"], rel=0.5)
    assert _flat_pixels(0, 0, p, R, frames=[(8, 4), (8, 2)]).square_steps() is None
    small = _tiles(2e-9, 6e-8)
    lv, info = engine.pixel_grouping(small, pix, k, 1e-6)
    assert lv == 4 and info["square_cross_rad"] < 1e-6 and info["square_tile_fraction"] == 1.0
    assert info["square_cross_rad"] > info["octet_cross_rad"]
    assert info["square_radius_m"] < info["octet_radius_m"]
    # tiles between the two radii: octets; a few of them among narrow
    # tiles: squares (the wide ones take the quad form inside the kernel)
    r_mid = 0.5 * (info["square_radius_m"] + info["octet_radius_m"])
    mid = _tiles(r_mid, 6e-8)
    lv, inf = engine.pixel_grouping(mid, pix, k, 1e-6)
    assert lv == 3 and inf["square_tile_fraction"] == 0.0
    mixed = _tiles(0, 6e-8, radii=[2e-9] * 7 + [r_mid])
    lv, inf = engine.pixel_grouping(mixed, pix, k, 1e-6)
    assert lv == 4 and inf["square_tile_fraction"] == pytest.approx(7 / 8)
    assert engine.pixel_grouping(small, pix, k, 1e-6, analyser=1)[0] == 2
    # the radius scales with the budget, the |d|^2 term's change counts
    r1 = engine.square_bounds(small, pix, k, 1e-6)["radius_m"]
    r2 = engine.square_bounds(small, pix, k, 2e-6)["radius_m"]
    assert r2 == pytest.approx(2 * r1, rel=1e-9)
    c0 = engine.square_bounds(small, pix, k, 1e-6)["cross"]
    c1 = engine.square_bounds(small, pix, k, 1e-6, fresnel_rad=1e-3)["cross"]
    assert c1 == pytest.approx(c0 + 4e-3 * st["extent"], rel=1e-9)


def test_square_steps_match_the_kernel_model():
    """square_steps' residual is the departure from exactly the model the
    kernel uses: mean of the 16 directions plus offsets times the means of
    the within-quad steps (columns 0->1, 2->3; rows 0->1, 2->3)."""
    p, R = 55e-6, 0.3
    pix = _flat_pixels(8, 4, p, R, y0=0.02, z0=0.05)
    u = (pix.xyz / torch.linalg.vector_norm(pix.xyz, dim=1, keepdim=True)).numpy()
    worst = 0.0
    U = u.reshape(4, 8, 3)
    for sq in range(2):
        B = U[:, 4 * sq:4 * sq + 4]                  # rows x columns x 3
        quads = [B[2 * (j >> 1):2 * (j >> 1) + 2, 2 * (j & 1):2 * (j & 1) + 2] for j in range(4)]
        g = sum((q[0, 1] - q[0, 0]) + (q[1, 1] - q[1, 0]) for q in quads) / 8
        h = sum((q[1, 0] - q[0, 0]) + (q[1, 1] - q[0, 1]) for q in quads) / 8
        mean = B.reshape(-1, 3).mean(0)
        for r in range(4):
            for c in range(4):
                model = mean + (c - 1.5) * g + (r - 1.5) * h
                worst = max(worst, float(np.linalg.norm(B[r, c] - model)))
    assert pix.square_steps()["plane"] == pytest.approx(worst, rel=1e-9)


def test_square_launch_clamps():
    k = 2 * np.pi / 1.2398e-10
    pix = _flat_pixels(16, 16, 55e-6, 1.0)
    small = _tiles(2e-9, 6e-8)
    lv, info = engine.pixel_grouping(small, pix, k, 1e-6)
    assert lv == 4
    g = lambda cfg, level=lv: engine.grouping_launch(cfg, level, small, pix, k, info)
    cfg = g(dict(pix_per_thread=16, threads=128, pairs=4))
    assert cfg["pairs"] == 4 and cfg["pair_short_radius_m"] == info["quad_short_radius_m"]
    assert cfg["octet_radius_m"] == info["square_radius_m"] > 0
    assert g(dict(pix_per_thread=8, threads=128, pairs=3))["octet_radius_m"] == info["octet_radius_m"]
    # squares need 16 pixels and 128 or 192 threads; 16 pixels and 192
    # threads exist only as squares
    assert g(dict(pix_per_thread=8, threads=128, pairs=4))["pairs"] == 3
    assert g(dict(pix_per_thread=16, threads=192, pairs=4))["pairs"] == 4
    c = g(dict(pix_per_thread=16, threads=256, pairs=4))
    assert (c["pairs"], c["pix_per_thread"]) == (3, 8)
    c = g(dict(pix_per_thread=16, threads=192, pairs=4), 3)
    assert (c["pairs"], c["pix_per_thread"], c["threads"]) == (3, 8, 128)
    c = g(dict(pix_per_thread=16, threads=128, pairs=4), 2)
    assert (c["pairs"], c["pix_per_thread"]) == (2, 8)
    c = g(dict(pix_per_thread=16, threads=128, pairs=4), 1)
    assert (c["pairs"], c["pix_per_thread"]) == (1, 4)
    assert engine.default_launch(4, 512) == dict(pix_per_thread=16, threads=128, slices=0, pairs=4)
    assert engine.default_launch(4) == engine.default_launch(4, engine.DEFAULT_TILE_ATOMS)
    assert engine.default_launch(4, 1024)["pairs"] == 4
    assert engine.default_launch(4, 2048) == engine.default_launch(3)
    a = engine.analyser_launch(dict(pix_per_thread=16, threads=128, pairs=4))
    assert (a["pairs"], a["pix_per_thread"]) == (2, 8)


def test_factor_table_admission():
    """The per-(species, pixel) factor table needs 2 (|o| + r) / R0 below
    1e-6 and no remove_forward."""
    pix = _flat_pixels(16, 16, 55e-6, 1.0)
    phys = types.SimpleNamespace(remove_forward=0)
    assert engine.factor_table_ok(_tiles(2e-9, 6e-8), pix, phys)
    assert not engine.factor_table_ok(_tiles(2e-9, 6e-7), pix, phys)
    assert not engine.factor_table_ok(_tiles(4e-7, 2e-7), pix, phys)
    assert not engine.factor_table_ok(_tiles(2e-9, 6e-8), _flat_pixels(16, 16, 55e-6, 0.05), phys)
    assert not engine.factor_table_ok(_tiles(2e-9, 6e-8), pix, types.SimpleNamespace(remove_forward=1))
    assert not engine.factor_table_ok(types.SimpleNamespace(n_tiles=0), pix, phys)


@pytest.mark.parametrize("form", ["octet", "square"])
@pytest.mark.parametrize("dist,o_max", [(1.0, 6e-8), (0.5, 3e-8), (0.2, 1e-8)])
def test_group_bound_covers_the_dropped_phase(form, dist, o_max):
    """The phase the octet (2x4) and square (4x4) forms drop, measured in
    FP64 on a flat detector for atoms anywhere in tiles of the form's radius
    at tile origins up to o_max from the sample origin: the kernel's phase
    model -- the group's mean direction plus the pixel offsets times the
    means of its quads' within-quad steps, the directions taken to each tile
    origin -- against the exact 2 pi D.(b - u'(P)) of every pixel, u'(P) the
    unit vector from the tile origin to the pixel. It stays within the
    bound's cross term for that radius (``octet_bounds``, ``square_bounds``)."""
    k = 2 * np.pi / 1.2398e-10
    kappa = k / (2 * np.pi)
    p = 55e-6
    gr, gc = (2, 4) if form == "octet" else (4, 4)
    bounds = engine.octet_bounds if form == "octet" else engine.square_bounds
    rng = np.random.default_rng(9)
    pix = _flat_pixels(16, 16, p, dist, y0=0.4 * dist, z0=0.2 * dist)
    r = bounds(_tiles(1e-9, o_max), pix, k, 1e-6)["radius_m"]
    bound = bounds(_tiles(r, o_max), pix, k, 1e-6)["cross"]
    assert bound <= 1e-6 * (1 + 1e-9)
    P = pix.xyz.numpy().reshape(16, 16, 3)          # rows x columns x 3
    b = np.array([1.0, 0.0, 0.0])
    worst = 0.0
    for _ in range(6):
        o = rng.standard_normal(3)
        o *= o_max * rng.uniform(0.5, 1.0) / np.linalg.norm(o)
        d = rng.standard_normal((64, 3))
        d *= (r * rng.uniform(0.0, 1.0, (64, 1)) ** (1 / 3)) / np.linalg.norm(d, axis=1, keepdims=True)
        U = P - o
        U /= np.linalg.norm(U, axis=-1, keepdims=True)
        W = b - U                                   # w of every pixel for this tile
        for r0 in range(0, 16, gr):
            for c0 in range(0, 16, gc):
                S = W[r0:r0 + gr, c0:c0 + gc]       # one octet or square
                quads = [S[i:i + 2, j:j + 2] for i in range(0, gr, 2) for j in range(0, gc, 2)]
                nq = len(quads)
                g = sum((q[0, 1] - q[0, 0]) + (q[1, 1] - q[1, 0]) for q in quads) / (2 * nq)
                h = sum((q[1, 0] - q[0, 0]) + (q[1, 1] - q[0, 1]) for q in quads) / (2 * nq)
                mean = S.reshape(-1, 3).mean(0)
                co = np.arange(gc) - (gc - 1) / 2
                ro = np.arange(gr) - (gr - 1) / 2
                model = mean + co[None, :, None] * g + ro[:, None, None] * h
                diff = (S - model).reshape(-1, 3)
                worst = max(worst, float(np.abs(2 * np.pi * kappa * d @ diff.T).max()))
    assert 0.0 < worst <= bound, (worst, bound)
