"""Analyser acceptance (the reference general kernel's top-hat / Darwin
factor, Beam.py:2350-2378) on the GPU: the FP64 plain kernel against the
oracle's double-precision restatement, the FP32 split kernel against both,
and the entry point's analyser axis (origin -> detector centre pixel,
Beam.py:6127-6131).

The reference evaluates the acceptance angle in float32 from cos(theta),
which near theta ~ 1e-3 rad resolves angles only to ~1e-5 rad; here (oracle
and kernels alike) theta comes from the chord |r_hat - c|, exact to
round-off, so that the edge of the acceptance is a property of the geometry.
"""
import numpy as np
import pytest

from mosaic_gb300 import Detector, StaticStage, engine, workloads
from mosaic_gb300.sample import ChunkedSample

import oracle
from helpers import field, rel_intensity, rel_max

pytestmark = pytest.mark.gpu


def _setup(shape=(24, 20), pitch=5.5e5):
    rng = np.random.default_rng(7)
    w = workloads.fcc_cu_32k(cells=8, npix=20)
    pos = w.sample.load_chunk_positions(1)
    spc = rng.choice(np.array(["Cu", "Ni"]), size=pos.shape[0])
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    D = Detector()
    D.create_detector(shape, (pitch, pitch))
    D.position_detector_absolute(2.0e9, 2.0 * w.meta["theta_deg"], 0.0)
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    return B, ChunkedSample([(pos, spc)]), D, stage, pos, spc


def _oracle(B, D, stage, pos, spc, analyser):
    return oracle.interact_cpu([(pos, spc)], D.pixel_coordinates, D.shape, stage.rotation,
                               stage.translation, B._energy, B.tables.f0,
                               {e: B.tables.f0_zero(e) for e in ("Cu", "Ni")}, B.tables.f1f2,
                               B._beam_E0_map, B._beam_grid(), B._polarization_state(),
                               apply_polarization=True, spherical_decay=True,
                               analyser=analyser).reshape(-1)


def _axis(D):
    ny, nz = D.shape
    c = np.asarray(D.pixel_coordinates)[:, (nz // 2) * ny + ny // 2]
    return (c.astype(np.float32) / np.float32(1e10)).astype(np.float64)


@pytest.mark.parametrize("mode,accept,hw", [("top-hat", 1.5e-3, 0.0), ("darwin", 0.0, 2e-3)])
def test_analyser_entry_point_matches_oracle(cuda, mode, accept, hw):
    B, sample, D, stage, pos, spc = _setup()
    kw = dict(apply_polarization=True, spherical_decay=True, return_double=True,
              analyser_mode=mode, analyser_acceptance_angle_rad=accept,
              analyser_darwin_halfwidth_rad=hw)
    kind = engine.analyser_kind(mode)
    ref = _oracle(B, D, stage, pos, spc, (kind, _axis(D), accept, hw))
    outs = {}
    for fast in (False, True):
        B._use_fast_kernel = fast
        outs[fast] = B.atomic_scattering_kinematic(sample, D, stage, **kw)
        assert B.last_run["path"] == ("split_f32" if fast else "plain_f64"), B.last_run
    # the analyser must bite: some pixels lose most of their intensity
    plain = _oracle(B, D, stage, pos, spc, None)
    ratio = np.abs(ref) ** 2 / np.maximum(np.abs(plain) ** 2, 1e-300)
    assert ratio.min() < 0.5 and ratio.max() > 0.5
    assert rel_max(outs[False].reshape(-1), ref) <= 1e-6, rel_max(outs[False].reshape(-1), ref)
    assert rel_intensity(outs[True].reshape(-1), ref) <= 1e-4, rel_intensity(outs[True].reshape(-1), ref)


def test_top_hat_edge_inside_tiles(cuda):
    """The acceptance edge put through one pixel: the half-angle is that
    pixel's angle from the axis as seen from the crystal's centre, so the edge
    cuts its atoms (and the tiles they sit in) about in half. The split
    kernel's per-atom edge test must match the oracle there, and that pixel
    must keep a fraction of its intensity strictly between 0 and 1."""
    B, sample, D, stage, pos, spc = _setup(shape=(33, 31))
    B._kernel_tile_atoms = 256
    ny, nz = D.shape
    coords = np.asarray(D.pixel_coordinates, np.float64) / 1e10
    p = (nz // 2 + 2) * ny + (ny // 2 + 3)
    lab = (np.asarray(pos, np.float32) @ np.asarray(stage.rotation, np.float32).T +
           np.asarray(stage.translation, np.float32)).astype(np.float64) / 1e10
    centre = lab.mean(0)
    axis = _axis(D)
    axis = axis / np.linalg.norm(axis)
    d = coords[:, p] - centre
    d /= np.linalg.norm(d)
    acc = 2.0 * np.arcsin(0.5 * np.linalg.norm(d - axis))
    kw = dict(apply_polarization=True, spherical_decay=True, return_double=True,
              analyser_mode="top-hat", analyser_acceptance_angle_rad=acc)
    ref = _oracle(B, D, stage, pos, spc, (1, _axis(D), acc, 0.0))
    plain = _oracle(B, D, stage, pos, spc, None)
    frac = abs(ref[p]) ** 2 / abs(plain[p]) ** 2
    assert 0.02 < frac < 0.98, frac
    B._use_fast_kernel = True
    got = B.atomic_scattering_kinematic(sample, D, stage, **kw).reshape(-1)
    assert B.last_run["path"] == "split_f32"
    assert rel_intensity(got, ref) <= 1e-4, rel_intensity(got, ref)
    assert abs(abs(got[p]) ** 2 - abs(ref[p]) ** 2) <= 1e-4 * abs(plain[p]) ** 2
    B._use_fast_kernel = False
    got64 = B.atomic_scattering_kinematic(sample, D, stage, **kw).reshape(-1)
    assert rel_max(got64, ref) <= 1e-6


def test_darwin_declines_when_too_narrow(cuda):
    """A Darwin width so narrow that the roll-off changes across a tile beyond
    the budget: the entry point declines to the FP64 kernel."""
    B, sample, D, stage, pos, spc = _setup()
    B._kernel_tile_atoms = 1024
    B._use_fast_kernel = True
    B.atomic_scattering_kinematic(sample, D, stage, analyser_mode="darwin",
                                  analyser_darwin_halfwidth_rad=1e-9, return_double=True)
    assert B.last_run["path"] == "plain_f64" and "analyser_err" in B.last_run


def test_analyser_launch_shapes(cuda):
    """The analyser kernels exist for 128/256 threads x 2/4 pixels (quads: x
    4/8 pixels): another shape is an argument error (never a silent drop of
    the analyser); the default shape runs."""
    from mosaic_gb300 import _lib
    B, sample, D, stage, pos, spc = _setup()
    atoms = B.stage_atoms(sample, stage)
    tiles = engine.Tiles(atoms, B.k, 256)
    phys = B.physics(True, True, False, analyser=(1, _axis(D), 1e-3, 0.0))
    pix = engine.Pixels(np.asarray(D.pixel_coordinates, np.float64) / 1e10, *D.shape, phys)
    with pytest.raises(ValueError):
        bad = dict(pix_per_thread=8, threads=64, slices=0)
        engine.run_split(tiles, pix, phys, atoms.table, launch=bad, fresnel=1)
    out = engine.run_split(tiles, pix, phys, atoms.table, fresnel=1)
    assert np.isfinite(field(out)).all()


@pytest.mark.parametrize("launch", [dict(pix_per_thread=8, threads=128),
                                    dict(pix_per_thread=4, threads=256)])
def test_top_hat_runs_quads(cuda, launch):
    """With a top-hat analyser the warps whose pixels take one factor per tile
    run the 2x2 quad form, those the edge cuts the per-atom loop: the result
    matches the oracle and one sin/cos per term (odd detector sides, so the
    ragged edge quads are in it too); a Darwin analyser shares nothing."""
    B, sample, D, stage, pos, spc = _setup(shape=(33, 31))
    B._kernel_tile_atoms = 256
    acc = 1.2e-3
    kw = dict(apply_polarization=True, spherical_decay=True, return_double=True,
              analyser_mode="top-hat", analyser_acceptance_angle_rad=acc)
    ref = _oracle(B, D, stage, pos, spc, (1, _axis(D), acc, 0.0))
    plain = _oracle(B, D, stage, pos, spc, None)
    ratio = np.abs(ref) ** 2 / np.maximum(np.abs(plain) ** 2, 1e-300)
    assert ratio.min() < 0.5 and ratio.max() > 0.5
    B._use_fast_kernel = True
    B._kernel_launch = dict(launch, slices=0, pairs=2)
    got = B.atomic_scattering_kinematic(sample, D, stage, **kw).reshape(-1)
    assert B.last_run["path"] == "split_f32" and B.last_run["launch"]["pairs"] == 2, B.last_run
    B._kernel_launch = dict(pix_per_thread=4, threads=128, slices=0, pairs=0)
    one = B.atomic_scattering_kinematic(sample, D, stage, **kw).reshape(-1)
    assert B.last_run["launch"]["pairs"] == 0
    assert rel_intensity(got, ref) <= 1e-4, rel_intensity(got, ref)
    assert rel_max(got, one) <= 2e-5, rel_max(got, one)
    B._kernel_launch = dict(launch, slices=0, pairs=2)
    B.atomic_scattering_kinematic(sample, D, stage, apply_polarization=True, spherical_decay=True,
                                  analyser_mode="darwin", analyser_darwin_halfwidth_rad=2e-3)
    assert B.last_run["launch"]["pairs"] == 0, B.last_run
