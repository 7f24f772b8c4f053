"""GPU parity of the 2x2 pixel-quad form (one sin/cos for four neighbouring
pixels): against the CPU oracle at the accuracy target (1e-4 relative
intensity), and against one sin/cos per term at 2e-5 of max |A| (the
truncated polynomials and the dropped mixed difference are each below
~2e-6 rad; the rest is FP32 rounding of two different summation orders)."""
import numpy as np
import pytest

from mosaic_gb300 import Detector, StaticStage, engine, workloads
from mosaic_gb300.sample import ChunkedSample
from mosaic_gb300.scan import BatchedScan, frames_from_motors

import oracle
from helpers import (atoms_from_arrays, field, kernel_case, oracle_case, rel_intensity, rel_max,
                     table_from_rows)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pix_pt,threads", [(4, 128), (8, 64), (4, 256), (8, 128)])
def test_split_quads_match_oracle(cuda, golden, pix_pt, threads):
    """The reference's kernel cases with an even detector (10 x 10 pixels,
    complex incident amplitudes: the complex-amplitude kernel)."""
    d = golden("kernel_cases.npz")
    used = 0
    for i in range(int(d["n"])):
        c = kernel_case(d, i)
        table, idx = table_from_rows(c["wk"], c["f0z"], c["anom"])
        atoms = atoms_from_arrays(c["pos"], idx, c["amp"], table, cuda)
        phys = engine.physics(c["k"], (1, 0, 0), c["ap"], c["pol"], c["dc"], c["rf"])
        pix = engine.Pixels(c["cxyz"], c["ny"], c["nz"], phys, device=cuda)
        tiles = engine.Tiles(atoms, c["k"], 128, device=cuda)
        level, info = engine.pixel_grouping(tiles, pix, c["k"], 1e-6)
        if level < 2:
            assert c["ny"] % 2 or c["nz"] % 2, (i, info)
            continue
        used += 1
        base = dict(pix_per_thread=pix_pt, threads=threads, slices=0)
        got = field(engine.run_split(tiles, pix, phys, table, fresnel=1, launch=dict(base, pairs=2)))
        one = field(engine.run_split(tiles, pix, phys, table, fresnel=1, launch=base))
        ref = oracle_case(c)
        assert rel_intensity(got, ref) <= 1e-4, (i, rel_intensity(got, ref))
        assert rel_max(got, ref) <= 1e-4, (i, rel_max(got, ref))
        assert rel_max(got, one) <= 2e-5, (i, rel_max(got, one))
    assert used >= 6


def test_quads_direct_sincos_argument(cuda, golden):
    """Tiles whose in-tile phase bound stays below the limit hand the phase
    to the sin/cos without the mod-1 reduction: the limit forced up (every
    short, |d|^2-free tile), the default (100 rad) and off agree with the
    oracle and with each other (the skipped reduction adds at most ~1e-7 |x|
    of phase per term, varying from atom to atom)."""
    d = golden("kernel_cases.npz")
    used = 0
    for i in range(int(d["n"])):
        c = kernel_case(d, i)
        if c["ny"] % 2 or c["nz"] % 2:
            continue
        table, idx = table_from_rows(c["wk"], c["f0z"], c["anom"])
        atoms = atoms_from_arrays(c["pos"], idx, c["amp"], table, cuda)
        phys = engine.physics(c["k"], (1, 0, 0), c["ap"], c["pol"], c["dc"], c["rf"])
        pix = engine.Pixels(c["cxyz"], c["ny"], c["nz"], phys, device=cuda)
        tiles = engine.Tiles(atoms, c["k"], 128, device=cuda)
        used += 1
        base = dict(pix_per_thread=4, threads=128, slices=0, pairs=2)
        run = lambda lim: field(engine.run_split(tiles, pix, phys, table, fresnel=0,
                                                 launch=dict(base, sin_direct_max_rad=lim)))
        always, default, never = run(1e4), run(0.0), run(-1.0)
        ref = oracle_case(c)
        for got in (always, default, never):
            assert rel_intensity(got, ref) <= 1e-4, (i, rel_intensity(got, ref))
        assert rel_max(always, never) <= 2e-5, (i, rel_max(always, never))
        assert rel_max(default, never) <= 2e-5, (i, rel_max(default, never))
    assert used >= 6


def _cu_ni_case():
    rng = np.random.default_rng(5)
    w = workloads.fcc_cu_32k(cells=8, npix=20)
    pos = w.sample.load_chunk_positions(1)
    spc = rng.choice(np.array(["Cu", "Ni"]), size=pos.shape[0])
    return w, pos, spc


def _det(shape, pitch, theta_deg):
    D = Detector()
    D.create_detector(shape, (pitch, pitch))
    D.position_detector_absolute(2.0e9, 2.0 * theta_deg, 0.0)
    return D


@pytest.mark.parametrize("shape,complex_beam", [((24, 20), False), ((16, 16), True)])
def test_split_quads_near_the_bound(cuda, shape, complex_beam):
    """A Cu/Ni crystal seen by a detector whose pitch puts the quad half
    differences at about 0.35 rad (0.5 is the limit: the long polynomials),
    through the entry point, which picks the quad form itself; with a
    complex incident wavefield too. A pitch that coarse (about 1 mm at
    0.2 m) makes the dropped mixed difference ~1e-5 rad, so the kernel phase
    budget is widened to 1e-4 rad (the reference's own knob) and the
    comparison with one sin/cos per term allows that dropped phase."""
    w, pos, spc = _cu_ni_case()
    sample = ChunkedSample([(pos, spc)])
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    B._kernel_phase_tol_rad = 1e-4
    if complex_beam:
        rng = np.random.default_rng(2)
        E0 = B._beam_E0_map * np.exp(1j * rng.uniform(-np.pi, np.pi, B._beam_E0_map.shape))
        B.set_wavefield(E0.astype(np.complex64))
    B._kernel_tile_atoms = 256
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    th = w.meta["theta_deg"]
    kw = dict(apply_polarization=True, spherical_decay=True, remove_forward=False, return_double=True)
    B._kernel_launch = dict(pix_per_thread=4, threads=128, slices=0, pairs=2)
    B.atomic_scattering_kinematic(sample, _det(shape, 5.5e5, th), stage, **kw)
    q0 = B.last_run["quad_delta_rad"]
    D = _det(shape, 5.5e5 * 0.35 / q0, th)
    got = B.atomic_scattering_kinematic(sample, D, stage, **kw)
    run = dict(B.last_run)
    assert run["path"] == "split_f32" and run["launch"]["pairs"] == 2, run
    assert 0.2 < run["quad_delta_rad"] <= engine.PAIR_DELTA_MAX, run["quad_delta_rad"]
    assert run["quad_cross_rad"] <= 1e-4, run["quad_cross_rad"]
    B._kernel_launch = dict(pix_per_thread=4, threads=128, slices=0, pairs=0)
    one = B.atomic_scattering_kinematic(sample, D, stage, **kw)
    ref = oracle.interact_cpu([(pos, spc)], D.pixel_coordinates, D.shape, stage.rotation,
                              stage.translation, B._energy, B.tables.f0,
                              {e: B.tables.f0_zero(e) for e in ("Cu", "Ni")}, B.tables.f1f2,
                              B._beam_E0_map, B._beam_grid(), B._polarization_state(),
                              apply_polarization=True, spherical_decay=True)
    assert rel_intensity(got, ref) <= 1e-4, rel_intensity(got, ref)
    assert rel_max(got, one) <= 2e-5 + run["quad_cross_rad"], (rel_max(got, one), run)


@pytest.mark.parametrize("shape,pix_pt", [((24, 21), 8), ((15, 12), 4), ((13, 11), 8),
                                           ((1, 7), 4), ((7, 1), 8), ((1, 1), 4)])
def test_quads_on_odd_detectors(cuda, shape, pix_pt):
    """Odd row lengths and odd numbers of rows (and single rows/columns): the
    quad at the ragged edge repeats its pixel, computes it twice and stores it
    once. The entry point picks quads itself (pairs are illegal when a pair
    would span a row end); every pixel matches the oracle and one sin/cos per
    term."""
    w, pos, spc = _cu_ni_case()
    sample = ChunkedSample([(pos, spc)])
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    B._kernel_tile_atoms = 256
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    D = _det(shape, 5.5e5, w.meta["theta_deg"])
    kw = dict(apply_polarization=True, spherical_decay=True, return_double=True)
    B._kernel_launch = dict(pix_per_thread=pix_pt, threads=128, slices=0, pairs=2)
    got = B.atomic_scattering_kinematic(sample, D, stage, **kw)
    assert B.last_run["launch"]["pairs"] == 2, B.last_run
    B._kernel_launch = dict(pix_per_thread=4, threads=128, slices=0, pairs=0)
    one = B.atomic_scattering_kinematic(sample, D, stage, **kw)
    ref = oracle.interact_cpu([(pos, spc)], D.pixel_coordinates, D.shape, stage.rotation,
                              stage.translation, B._energy, B.tables.f0,
                              {e: B.tables.f0_zero(e) for e in ("Cu", "Ni")}, B.tables.f1f2,
                              B._beam_E0_map, B._beam_grid(), B._polarization_state(),
                              apply_polarization=True, spherical_decay=True)
    assert got.shape == ref.shape == (shape[1], shape[0])
    assert rel_intensity(got, ref) <= 1e-4, rel_intensity(got, ref)
    assert rel_max(got, one) <= 2e-5, rel_max(got, one)


def _scan_frames(rois):
    w = workloads.fcc_cu_32k(cells=10, npix=64)
    theta = np.radians(w.meta["theta_deg"])
    steps = [dict(mu=theta + np.radians(d), chi=np.radians(c))
             for c in (-0.4, 0.3) for d in (-1.0, 0.0, 0.5)]
    return w, frames_from_motors(w.stage, w.detector, steps, rois)


def test_scan_quads_match_pairs_and_single_exposures(cuda):
    """A batched scan over ROIs of uneven (even) sides runs the quad form;
    every frame matches the pair form and FP64 single exposures."""
    w, frames = _scan_frames([16, 64, 24, 8, 40, 32])
    B = w.beam
    quad = BatchedScan(B, w.sample, frames, launch=dict(pix_per_thread=8, threads=128, pairs=2),
                       **w.sc_kwargs)
    assert quad.cfg["pairs"] == 2, quad.cfg
    quad.run()
    pair = BatchedScan(B, w.sample, frames, launch=dict(pairs=1), **w.sc_kwargs)
    assert pair.cfg["pairs"] == 1
    pair.run()
    B._use_fast_kernel = False
    for f, fr in enumerate(frames):
        got, alt = quad.frame_field(f), pair.frame_field(f)
        assert rel_max(got, alt) <= 2e-5, (f, rel_max(got, alt))
        ref = B.interact_beam_gpu(w.sample, fr.pixels, fr.shape,
                                  StaticStage(fr.rotation, fr.translation), apply_polarization=True,
                                  spherical_decay=False, return_double=True)
        assert rel_intensity(got, ref) <= 1e-4, (f, rel_intensity(got, ref))


def test_scan_with_odd_rois_runs_quads(cuda):
    """ROIs of odd side in one batched launch: quads with repeated edge
    pixels, every frame equal to the pair-free form."""
    w, frames = _scan_frames([16, 15, 9, 8, 1, 33])
    B = w.beam
    quad = BatchedScan(B, w.sample, frames, **w.sc_kwargs)
    assert quad.cfg["pairs"] == 2, quad.cfg
    quad.run()
    one = BatchedScan(B, w.sample, frames, launch=dict(pairs=0), **w.sc_kwargs)
    assert one.cfg["pairs"] == 0
    one.run()
    for f in range(len(frames)):
        got, alt = quad.frame_field(f), one.frame_field(f)
        assert rel_max(got, alt) <= 2e-5, (f, rel_max(got, alt))
