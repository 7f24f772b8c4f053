"""The 4x4 pixel-square form of the split kernel (four 2x2 quads sharing
their half differences) against the oracle, the octet and quad forms and
one sin/cos per term.

Tolerances: 1e-4 relative intensity against the oracle (the FP32 path's
gate); 2e-5 of max |A| against the other forms (the budget of the quad and
octet forms' tests), plus the dropped phase the host bounds when the test
widens the phase budget.
"""
import numpy as np
import pytest

import oracle
from helpers import rel_intensity, rel_max
from mosaic_gb300 import Detector, StaticStage, engine, workloads
from mosaic_gb300.sample import ChunkedSample
from mosaic_gb300.scan import BatchedScan, frames_from_motors

pytestmark = pytest.mark.gpu

SQ = dict(pix_per_thread=16, threads=128, slices=0, pairs=4)
OCT = dict(pix_per_thread=8, threads=128, slices=0, pairs=3)
QUAD = dict(pix_per_thread=8, threads=128, slices=0, pairs=2)
ONE = dict(pix_per_thread=4, threads=128, slices=0, pairs=0)


def _cu_ni_case():
    rng = np.random.default_rng(5)
    w = workloads.fcc_cu_32k(cells=8, npix=20)
    pos = w.sample.load_chunk_positions(1)
    spc = rng.choice(np.array(["Cu", "Ni"]), size=pos.shape[0])
    return w, pos, spc


def _det(shape, pitch, theta_deg, dist=1.0e10):
    D = Detector()
    D.create_detector(shape, (pitch, pitch))
    D.position_detector_absolute(dist, 2.0 * theta_deg, 0.0)
    return D


def _oracle(B, pos, spc, D, stage):
    return oracle.interact_cpu([(pos, spc)], D.pixel_coordinates, D.shape, stage.rotation,
                               stage.translation, B._energy, B.tables.f0,
                               {e: B.tables.f0_zero(e) for e in ("Cu", "Ni")}, B.tables.f1f2,
                               B._beam_E0_map, B._beam_grid(), B._polarization_state(),
                               apply_polarization=True, spherical_decay=True)


def _staged(B, pos, spc, D, stage, cuda, tile_atoms):
    phys = B.physics(apply_polarization=True, spherical_decay=True)
    atoms = B.stage_atoms(ChunkedSample([(pos, spc)]), stage, device=cuda)
    tiles = engine.Tiles(atoms, B.k, tile_atoms, device=cuda)
    pix = engine.Pixels(np.asarray(D.pixel_coordinates, np.float64) / 1e10, *D.shape, phys,
                        device=cuda)
    return phys, atoms, tiles, pix


@pytest.mark.parametrize("shape,threads,complex_beam", [((24, 20), 128, False), ((16, 16), 192, True),
                                                         ((32, 8), 128, False), ((4, 4), 192, False)])
def test_squares_match_oracle_and_other_forms(cuda, shape, threads, complex_beam):
    """A Cu/Ni crystal at its (111) reflection, 1 m, through the entry
    point: squares on detectors of whole squares (the smallest one a single
    square), 128- and 192-thread blocks, with a complex incident wavefield
    too."""
    w, pos, spc = _cu_ni_case()
    sample = ChunkedSample([(pos, spc)])
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    if complex_beam:
        rng = np.random.default_rng(2)
        E0 = B._beam_E0_map * np.exp(1j * rng.uniform(-np.pi, np.pi, B._beam_E0_map.shape))
        B.set_wavefield(E0.astype(np.complex64))
    B._kernel_tile_atoms = 256
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    D = _det(shape, 5.5e5, w.meta["theta_deg"])
    kw = dict(apply_polarization=True, spherical_decay=True, return_double=True)
    out = {}
    for name, cfg in (("sq", dict(SQ, threads=threads)), ("oct", OCT), ("quad", QUAD), ("one", ONE)):
        B._kernel_launch = cfg
        out[name] = B.atomic_scattering_kinematic(sample, D, stage, **kw)
        assert B.last_run["launch"]["pairs"] == cfg["pairs"], (name, B.last_run)
        if name == "sq":
            assert B.last_run["square_cross_rad"] <= 1e-6, B.last_run
            assert B.last_run["square_tile_fraction"] == 1.0, B.last_run
            assert B.last_run["launch"]["octet_radius_m"] == B.last_run["square_radius_m"]
    ref = _oracle(B, pos, spc, D, stage)
    assert rel_intensity(out["sq"], ref) <= 1e-4, rel_intensity(out["sq"], ref)
    assert rel_max(out["sq"], ref) <= 1e-4, rel_max(out["sq"], ref)
    for other in ("oct", "quad", "one"):
        assert rel_max(out["sq"], out[other]) <= 2e-5, (other, rel_max(out["sq"], out[other]))


def test_squares_direct_sincos_argument(cuda):
    """The direct sin/cos argument forced on for every short tile, at the
    default limit and off: all agree with the oracle and with each other."""
    w, pos, spc = _cu_ni_case()
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    D = _det((24, 20), 5.5e5, w.meta["theta_deg"])
    phys, atoms, tiles, pix = _staged(B, pos, spc, D, stage, cuda, 256)
    level, info = engine.pixel_grouping(tiles, pix, B.k, 1e-6)
    assert level == 4, info

    def run(lim):
        cfg = dict(SQ, sin_direct_max_rad=lim, pair_short_radius_m=info["quad_short_radius_m"],
                   octet_radius_m=info["square_radius_m"])
        o = engine.run_split(tiles, pix, phys, atoms.table, launch=cfg, fresnel=0)
        engine.sync()
        return o.cpu().numpy()

    always, default, never = run(1e4), run(0.0), run(-1.0)
    c = lambda a: (a[:, 0] + 1j * a[:, 1]).reshape(D.shape[1], D.shape[0])
    ref = _oracle(B, pos, spc, D, stage)
    for got in (always, default, never):
        assert rel_intensity(c(got), ref) <= 1e-4, rel_intensity(c(got), ref)
    assert rel_max(always, never) <= 2e-5, rel_max(always, never)
    assert rel_max(default, never) <= 2e-5, rel_max(default, never)


def test_squares_with_wide_tiles_taking_quads(cuda):
    """The square kernel switches to the quad form per tile: with the
    square radius at the median tile radius about half the tiles take each
    form, and the result equals the all-square and the all-quad runs
    (within the forms' budget) and the oracle; with radius 0 every tile
    takes the quad arithmetic of the 8-pixel quad kernel."""
    w, pos, spc = _cu_ni_case()
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    D = _det((24, 20), 5.5e5, w.meta["theta_deg"])
    phys, atoms, tiles, pix = _staged(B, pos, spc, D, stage, cuda, 128)
    level, info = engine.pixel_grouping(tiles, pix, B.k, 1e-6)
    assert level == 4, info
    radii = tiles.origin[: tiles.n_tiles, 3].cpu().numpy()
    assert tiles.n_tiles >= 8 and radii.max() <= info["square_radius_m"]
    med = float(np.median(radii))
    assert 0.2 < float((radii <= med).mean()) < 0.8

    def run(cfg):
        cfg = dict(cfg, pair_short_radius_m=info["quad_short_radius_m"])
        o = engine.run_split(tiles, pix, phys, atoms.table, launch=cfg, fresnel=0)
        engine.sync()
        a = o.cpu().numpy()
        return (a[:, 0] + 1j * a[:, 1]).reshape(D.shape[1], D.shape[0])

    mixed = run(dict(SQ, octet_radius_m=med))
    all_sq = run(dict(SQ, octet_radius_m=info["square_radius_m"]))
    all_quad = run(dict(SQ, octet_radius_m=0.0))
    quads = run(QUAD)
    assert rel_max(all_quad, quads) <= 1e-6         # the same quad arithmetic per tile
    assert rel_max(mixed, all_sq) <= 2e-5 and rel_max(mixed, quads) <= 2e-5
    assert rel_intensity(mixed, _oracle(B, pos, spc, D, stage)) <= 1e-4


def test_squares_with_the_fresnel_term(cuda):
    """Tiles that keep the |d|^2 term (at 0.2 m, every tile wider than the
    Fresnel radius), the long polynomials (the short radius set to 0) and
    the mod-1 reduction (direct argument off): squares against one sin/cos
    per term and the oracle, the budget widened to 1e-4 rad so that the
    host admits squares."""
    w, pos, spc = _cu_ni_case()
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    D = _det((16, 16), 5.5e5, w.meta["theta_deg"], dist=2.0e9)
    phys, atoms, tiles, pix = _staged(B, pos, spc, D, stage, cuda, 256)
    level, info = engine.pixel_grouping(tiles, pix, B.k, 1e-4)
    assert level == 4, info

    def run(cfg):
        o = engine.run_split(tiles, pix, phys, atoms.table, launch=cfg, fresnel=1)
        engine.sync()
        a = o.cpu().numpy()
        return (a[:, 0] + 1j * a[:, 1]).reshape(D.shape[1], D.shape[0])

    sq = run(dict(SQ, pair_short_radius_m=0.0, sin_direct_max_rad=-1.0,
                  octet_radius_m=info["square_radius_m"]))
    one = run(ONE)
    ref = _oracle(B, pos, spc, D, stage)
    assert rel_intensity(sq, ref) <= 1e-4, rel_intensity(sq, ref)
    assert rel_max(sq, one) <= 2e-5 + info["square_cross_rad"], (rel_max(sq, one), info)


def test_squares_declined_on_shapes_that_are_not_whole_squares(cuda):
    """A row count that is not a multiple of 4 keeps octets (whole octets)
    or quads; the planner refuses a square plan there."""
    w, pos, spc = _cu_ni_case()
    sample = ChunkedSample([(pos, spc)])
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    B._kernel_tile_atoms = 256
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    B._kernel_launch = SQ
    for shape, mode in (((24, 18), 3), ((22, 20), 2), ((7, 3), 2)):
        D = _det(shape, 5.5e5, w.meta["theta_deg"])
        got = B.atomic_scattering_kinematic(sample, D, stage, return_double=True,
                                            apply_polarization=True, spherical_decay=True)
        assert B.last_run["launch"]["pairs"] == mode, (shape, B.last_run)
        ref = _oracle(B, pos, spc, D, stage)
        assert rel_intensity(got, ref) <= 1e-4, (shape, rel_intensity(got, ref))
    D = _det((24, 18), 5.5e5, w.meta["theta_deg"])
    phys, atoms, tiles, pix = _staged(B, pos, spc, D, stage, cuda, 256)
    with pytest.raises(ValueError):
        engine.run_split(tiles, pix, phys, atoms.table, launch=dict(SQ, pair_short_radius_m=0.0))


def test_scan_squares_match_octets_and_single_exposures(cuda):
    """A batched scan over ROIs of sides that are multiples of 4 runs the
    square form; every frame matches the octet form and FP64 single
    exposures."""
    w = workloads.fcc_cu_32k(cells=10, npix=64)
    theta = np.radians(w.meta["theta_deg"])
    steps = [dict(mu=theta + np.radians(d), chi=np.radians(c))
             for c in (-0.4, 0.3) for d in (-1.0, 0.0, 0.5)]
    frames = frames_from_motors(w.stage, w.detector, steps, [16, 64, 24, 8, 40, 32])
    B = w.beam
    sqs = BatchedScan(B, w.sample, frames, launch=SQ, **w.sc_kwargs)
    assert sqs.cfg["pairs"] == 4, sqs.cfg
    sqs.run()
    octs = BatchedScan(B, w.sample, frames, launch=OCT, staged=sqs, **w.sc_kwargs)
    assert octs.cfg["pairs"] == 3
    octs.run()
    B._use_fast_kernel = False
    for f, fr in enumerate(frames):
        got, alt = sqs.frame_field(f), octs.frame_field(f)
        assert rel_max(got, alt) <= 2e-5, (f, rel_max(got, alt))
        ref = B.interact_beam_gpu(w.sample, fr.pixels, fr.shape,
                                  StaticStage(fr.rotation, fr.translation), apply_polarization=True,
                                  spherical_decay=False, return_double=True)
        assert rel_intensity(got, ref) <= 1e-4, (f, rel_intensity(got, ref))
