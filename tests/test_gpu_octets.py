"""The 2x4 pixel-octet form of the split kernel (two 2x2 quads side by side
sharing their half differences) against the oracle, the quad form and one
sin/cos per term.

Tolerances: 1e-4 relative intensity against the oracle (the FP32 path's
gate); 2e-5 of max |A| against the other forms (the same budget as the quad
form's tests), plus the dropped phase the host bounds when the test widens
the phase budget.
"""
import numpy as np
import pytest

import oracle
from helpers import rel_intensity, rel_max
from mosaic_gb300 import Detector, StaticStage, engine, workloads
from mosaic_gb300.sample import ChunkedSample
from mosaic_gb300.scan import BatchedScan, frames_from_motors

pytestmark = pytest.mark.gpu

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


@pytest.mark.parametrize("shape,threads,complex_beam", [((24, 20), 128, False), ((16, 16), 64, True),
                                                         ((32, 6), 256, False), ((4, 2), 128, False)])
def test_octets_match_oracle_and_other_forms(cuda, shape, threads, complex_beam):
    """A Cu/Ni crystal at its (111) reflection, 1 m, through the entry
    point: octets on detectors of whole octets (the smallest one a single
    octet), with a complex incident wavefield too. (At 0.2 m the octet's
    dropped phase exceeds the 1e-6 rad budget for tiles of this size and the
    host keeps quads.)"""
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
    for name, cfg in (("oct", dict(OCT, threads=threads)), ("quad", QUAD), ("one", ONE)):
        B._kernel_launch = cfg
        out[name] = B.atomic_scattering_kinematic(sample, D, stage, **kw)
        assert B.last_run["launch"]["pairs"] == cfg["pairs"], (name, B.last_run)
        if name == "oct":
            assert B.last_run["octet_cross_rad"] <= 1e-6, B.last_run
            assert B.last_run["octet_tile_fraction"] == 1.0, B.last_run
    ref = _oracle(B, pos, spc, D, stage)
    assert rel_intensity(out["oct"], ref) <= 1e-4, rel_intensity(out["oct"], ref)
    assert rel_max(out["oct"], ref) <= 1e-4, rel_max(out["oct"], ref)
    assert rel_max(out["oct"], out["quad"]) <= 2e-5, rel_max(out["oct"], out["quad"])
    assert rel_max(out["oct"], out["one"]) <= 2e-5, rel_max(out["oct"], out["one"])


def test_octets_direct_sincos_argument(cuda):
    """The direct sin/cos argument forced on for every short tile, at the
    default limit and off: all agree with the oracle and with each other."""
    w, pos, spc = _cu_ni_case()
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    D = _det((24, 20), 5.5e5, w.meta["theta_deg"])
    phys = B.physics(apply_polarization=True, spherical_decay=True)
    atoms = B.stage_atoms(ChunkedSample([(pos, spc)]), stage, device=cuda)
    tiles = engine.Tiles(atoms, B.k, 256, device=cuda)
    pix = engine.Pixels(np.asarray(D.pixel_coordinates, np.float64) / 1e10, *D.shape, phys,
                        device=cuda)
    level, info = engine.pixel_grouping(tiles, pix, B.k, 1e-6)
    assert level >= 3, info
    short_r = info["quad_short_radius_m"]

    def run(lim):
        cfg = dict(OCT, sin_direct_max_rad=lim, pair_short_radius_m=short_r,
                   octet_radius_m=info["octet_radius_m"])
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


def test_octets_with_wide_tiles_taking_quads(cuda):
    """The octet kernel switches to the quad form per tile: with the octet
    radius at the median tile radius half the tiles take each form, and the
    result equals both the all-octet and the all-quad runs (within the
    forms' budget) and the oracle."""
    w, pos, spc = _cu_ni_case()
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    D = _det((24, 20), 5.5e5, w.meta["theta_deg"])
    phys = B.physics(apply_polarization=True, spherical_decay=True)
    atoms = B.stage_atoms(ChunkedSample([(pos, spc)]), stage, device=cuda)
    tiles = engine.Tiles(atoms, B.k, 128, device=cuda)
    pix = engine.Pixels(np.asarray(D.pixel_coordinates, np.float64) / 1e10, *D.shape, phys,
                        device=cuda)
    level, info = engine.pixel_grouping(tiles, pix, B.k, 1e-6)
    assert level >= 3, info
    radii = tiles.origin[: tiles.n_tiles, 3].cpu().numpy()
    assert tiles.n_tiles >= 8 and radii.max() <= info["octet_radius_m"]
    med = float(np.median(radii))
    assert 0.2 < float((radii <= med).mean()) < 0.8

    def run(cfg):
        cfg = dict(cfg, pair_short_radius_m=info["quad_short_radius_m"])
        o = engine.run_split(tiles, pix, phys, atoms.table, launch=cfg, fresnel=0)
        engine.sync()
        a = o.cpu().numpy()
        return (a[:, 0] + 1j * a[:, 1]).reshape(D.shape[1], D.shape[0])

    mixed = run(dict(OCT, octet_radius_m=med))
    all_oct = run(dict(OCT, octet_radius_m=info["octet_radius_m"]))
    all_quad = run(dict(OCT, octet_radius_m=0.0))
    quads = run(QUAD)
    assert rel_max(all_quad, quads) <= 1e-6         # the same quad arithmetic per tile
    assert rel_max(mixed, all_oct) <= 2e-5 and rel_max(mixed, quads) <= 2e-5
    assert rel_intensity(mixed, _oracle(B, pos, spc, D, stage)) <= 1e-4


def test_octets_near_the_bound(cuda):
    """A detector whose pitch puts the shared half differences at about
    0.35 rad (the long polynomials) and the octet's dropped phase near the
    widened 1e-4 rad budget: octets against the oracle and one sin/cos per
    term (which may differ by that dropped phase)."""
    w, pos, spc = _cu_ni_case()
    sample = ChunkedSample([(pos, spc)])
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    B._kernel_phase_tol_rad = 1e-4
    B._kernel_tile_atoms = 256
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    th = w.meta["theta_deg"]
    kw = dict(apply_polarization=True, spherical_decay=True, return_double=True)
    B._kernel_launch = OCT
    B.atomic_scattering_kinematic(sample, _det((24, 20), 5.5e5, th), stage, **kw)
    q0 = B.last_run["quad_delta_rad"]
    D = _det((24, 20), 5.5e5 * 0.35 / q0, th)
    got = B.atomic_scattering_kinematic(sample, D, stage, **kw)
    run = dict(B.last_run)
    if run["launch"]["pairs"] != 3:
        pytest.skip(f"octets not admitted at this pitch: {run.get('octet_cross_rad')}")
    assert 0.2 < run["quad_delta_rad"] <= engine.PAIR_DELTA_MAX, run
    B._kernel_launch = ONE
    one = B.atomic_scattering_kinematic(sample, D, stage, **kw)
    ref = _oracle(B, pos, spc, D, stage)
    assert rel_intensity(got, ref) <= 1e-4, rel_intensity(got, ref)
    assert rel_max(got, one) <= 2e-5 + run["octet_cross_rad"], (rel_max(got, one), run)


def test_octets_declined_on_shapes_that_are_not_whole_octets(cuda):
    """Rows not a multiple of 4 or an odd row count: the host keeps quads
    (an octet launch is clamped), and the planner refuses an octet plan."""
    w, pos, spc = _cu_ni_case()
    sample = ChunkedSample([(pos, spc)])
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    B._kernel_tile_atoms = 256
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    B._kernel_launch = OCT
    for shape in ((22, 20), (24, 19), (7, 3)):
        D = _det(shape, 5.5e5, w.meta["theta_deg"])
        got = B.atomic_scattering_kinematic(sample, D, stage, return_double=True,
                                            apply_polarization=True, spherical_decay=True)
        assert B.last_run["launch"]["pairs"] == 2, (shape, B.last_run)
        ref = _oracle(B, pos, spc, D, stage)
        assert rel_intensity(got, ref) <= 1e-4, (shape, rel_intensity(got, ref))
    phys = B.physics()
    atoms = B.stage_atoms(sample, stage, device=cuda)
    tiles = engine.Tiles(atoms, B.k, 256, device=cuda)
    D = _det((22, 20), 5.5e5, w.meta["theta_deg"])
    pix = engine.Pixels(np.asarray(D.pixel_coordinates, np.float64) / 1e10, *D.shape, phys,
                        device=cuda)
    with pytest.raises(ValueError):
        engine.run_split(tiles, pix, phys, atoms.table, launch=dict(OCT, pair_short_radius_m=0.0))


def test_scan_octets_match_quads_and_single_exposures(cuda):
    """A batched scan over ROIs of sides that are multiples of 4 runs the
    octet form; every frame matches the quad form and FP64 single
    exposures."""
    w = workloads.fcc_cu_32k(cells=10, npix=64)
    theta = np.radians(w.meta["theta_deg"])
    steps = [dict(mu=theta + np.radians(d), chi=np.radians(c))
             for c in (-0.4, 0.3) for d in (-1.0, 0.0, 0.5)]
    frames = frames_from_motors(w.stage, w.detector, steps, [16, 64, 24, 8, 40, 32])
    B = w.beam
    octs = BatchedScan(B, w.sample, frames, launch=OCT, **w.sc_kwargs)
    assert octs.cfg["pairs"] == 3, octs.cfg
    octs.run()
    quad = BatchedScan(B, w.sample, frames, launch=QUAD, staged=octs, **w.sc_kwargs)
    assert quad.cfg["pairs"] == 2
    quad.run()
    B._use_fast_kernel = False
    for f, fr in enumerate(frames):
        got, alt = octs.frame_field(f), quad.frame_field(f)
        assert rel_max(got, alt) <= 2e-5, (f, rel_max(got, alt))
        ref = B.interact_beam_gpu(w.sample, fr.pixels, fr.shape,
                                  StaticStage(fr.rotation, fr.translation), apply_polarization=True,
                                  spherical_decay=False, return_double=True)
        assert rel_intensity(got, ref) <= 1e-4, (f, rel_intensity(got, ref))
