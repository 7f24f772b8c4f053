"""GPU parity: the sm_103a kernels against the CPU oracle and the reference's
own outputs (golden fixtures made by running the reference).

Tolerances
  * FP64 plain vs the (uncontracted) FP64 oracle: 1e-12 of the largest |A|
    (same arithmetic; GPU and libm differ only in the last bit of sin/cos/exp).
  * FP64 plain vs the reference cffi kernel: 1e-5 of max |A| (that build
    contracts FMAs, which moves the ~1e10 rad absolute phase by ~1e-6 rad),
    vs its NumPy twin: 2e-7 (the reference rounds its output to float32).
  * FP32 split-phase vs FP64: 1e-4 relative intensity error
    max|I - I_ref| / max I_ref (the accuracy target), and 1e-4 of max |A|.
"""
import numpy as np
import pytest
import torch

from mosaic_gb300 import Detector, StaticStage, engine, workloads
from mosaic_gb300.beam import beam as Beam
from mosaic_gb300.sample import ChunkedSample

import oracle
from helpers import (atoms_from_arrays, field, kernel_case, oracle_case, rel_intensity, rel_max,
                     run_case, table_from_rows)

pytestmark = pytest.mark.gpu


def test_plain_f64_matches_oracle_and_reference(cuda, golden):
    d = golden("kernel_cases.npz")
    for i in range(int(d["n"])):
        c = kernel_case(d, i)
        got = run_case(c, cuda, fast=False)
        ref = oracle_case(c)
        assert rel_max(got, ref) <= 1e-12, (i, rel_max(got, ref))
        assert rel_max(got, c["numpy"]) <= 2e-7, (i, rel_max(got, c["numpy"]))
        assert rel_max(got, c["cffi"]) <= 1e-5, (i, rel_max(got, c["cffi"]))


@pytest.mark.parametrize("tile_atoms", [128, 256])
def test_split_f32_matches_oracle(cuda, golden, tile_atoms):
    d = golden("kernel_cases.npz")
    for i in range(int(d["n"])):
        c = kernel_case(d, i)
        got = run_case(c, cuda, fast=True, tile_atoms=tile_atoms)
        ref = oracle_case(c)
        assert rel_intensity(got, ref) <= 1e-4, (i, rel_intensity(got, ref))
        assert rel_max(got, ref) <= 1e-4, (i, rel_max(got, ref))


@pytest.mark.parametrize("pix_pt", [2, 4, 8])
def test_split_pairs_match_oracle(cuda, golden, pix_pt):
    """Pixel-pair form (one sin/cos for two neighbouring pixels) on the
    reference's kernel cases, wherever the pair bound admits it."""
    d = golden("kernel_cases.npz")
    used = 0
    for i in range(int(d["n"])):
        c = kernel_case(d, i)
        table, idx = table_from_rows(c["wk"], c["f0z"], c["anom"])
        atoms = atoms_from_arrays(c["pos"], idx, c["amp"], table, cuda)
        phys = engine.physics(c["k"], (1, 0, 0), c["ap"], c["pol"], c["dc"], c["rf"])
        pix = engine.Pixels(c["cxyz"], c["ny"], c["nz"], phys, device=cuda)
        tiles = engine.Tiles(atoms, c["k"], 128, device=cuda)
        if not engine.pairs_allowed(tiles, pix, c["k"]):
            continue
        used += 1
        base = dict(pix_per_thread=pix_pt, threads=128, slices=0)
        got = field(engine.run_split(tiles, pix, phys, table, fresnel=1, launch=dict(base, pairs=1)))
        one = field(engine.run_split(tiles, pix, phys, table, fresnel=1, launch=base))
        ref = oracle_case(c)
        assert rel_intensity(got, ref) <= 1e-4, (i, rel_intensity(got, ref))
        assert rel_max(got, ref) <= 1e-4, (i, rel_max(got, ref))
        assert rel_max(got, one) <= 2e-5, (i, rel_max(got, one))
    assert used >= 1


@pytest.mark.parametrize("shape", [(24, 20), (13, 11), (25, 1)])
def test_split_pairs_near_the_bound(cuda, shape):
    """A (111)-oriented fcc Cu/Ni crystal seen by a detector whose pitch puts
    the pair half-phase at about 0.35 rad (0.5 is the limit), odd pixel counts
    and odd rows included (the pair then spans a row end, or the last pixel
    pairs with itself): pair form against the oracle and against one sin/cos
    per term."""
    rng = np.random.default_rng(3)
    w = workloads.fcc_cu_32k(cells=8, npix=20)
    pos = w.sample.load_chunk_positions(1)
    spc = rng.choice(np.array(["Cu", "Ni"]), size=pos.shape[0])
    sample = ChunkedSample([(pos, spc)])
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    B._kernel_tile_atoms = 256
    stage = StaticStage(w.stage.rotation, w.stage.translation)

    def det(pitch):
        D = Detector()
        D.create_detector(shape, (pitch, pitch))
        D.position_detector_absolute(2.0e9, 2.0 * w.meta["theta_deg"], 0.0)
        return D

    kw = dict(apply_polarization=True, spherical_decay=True, remove_forward=False, return_double=True)
    B._kernel_launch = dict(pix_per_thread=4, threads=128, slices=0, pairs=1)
    B.atomic_scattering_kinematic(sample, det(5.5e5), stage, **kw)
    d0 = B.last_run["pair_delta_rad"]
    pitch = 5.5e5 * 0.35 / d0
    D = det(pitch)
    got = B.atomic_scattering_kinematic(sample, D, stage, **kw)
    run = dict(B.last_run)
    assert run["path"] == "split_f32" and run["launch"]["pairs"] == 1, run
    assert 0.2 < run["pair_delta_rad"] <= engine.PAIR_DELTA_MAX, run["pair_delta_rad"]
    B._kernel_launch = dict(pix_per_thread=4, threads=128, slices=0, pairs=0)
    one = B.atomic_scattering_kinematic(sample, D, stage, **kw)
    ref = oracle.interact_cpu([(pos, spc)], D.pixel_coordinates, D.shape, stage.rotation,
                              stage.translation, B._energy, B.tables.f0,
                              {e: B.tables.f0_zero(e) for e in ("Cu", "Ni")}, B.tables.f1f2,
                              B._beam_E0_map, B._beam_grid(), B._polarization_state(),
                              apply_polarization=True, spherical_decay=True)
    assert rel_intensity(got, ref) <= 1e-4, rel_intensity(got, ref)
    assert rel_max(got, one) <= 2e-5, rel_max(got, one)


def _golden_beam(e):
    B = Beam()
    B.create_beam(float(e["energy"]), beam_size=(70.0, 60.0), beam_samples=(64, 48),
                  beam_profile="gaussian", gaussian_waist=(30.0, 25.0), pol_perp_rate=0.9)
    # The Gaussian profile goes through np.exp, whose last bit differs between
    # libm builds (x86 vs Arm): use the reference's own map.
    assert np.allclose(B._beam_E0_map, e["E0"], rtol=1e-6, atol=0)
    B.set_wavefield(e["E0"])
    return B


@pytest.mark.parametrize("fast", [False, True])
def test_entry_point_matches_reference_interact_cpu(cuda, golden, fast):
    """beam.interact_beam_gpu on the reference's own end-to-end case (two
    chunks, three species, rotated + translated stage, Gaussian beam)."""
    e = golden("interact_cpu.npz")
    sample = ChunkedSample([(e["pos0"], e["spc0"]), (e["pos1"], e["spc1"])])
    stage = StaticStage(e["rotation"], e["translation"])
    B = _golden_beam(e)
    B._use_fast_kernel = fast
    shape = tuple(int(v) for v in e["shape"])
    for i in range(3):
        rf, ap, dc = (bool(v) for v in e[f"flags{i}"])
        got = B.interact_beam_gpu(sample, e["coords"], shape, stage, remove_forward=rf,
                                  apply_polarization=ap, spherical_decay=dc, return_double=True)
        assert B.last_run["path"] == ("split_f32" if fast else "plain_f64")
        ref = e[f"out{i}"]
        tol = 1e-4 if fast else 1e-5
        assert got.shape == ref.shape
        assert rel_intensity(got, ref) <= tol, (i, rel_intensity(got, ref))


def test_entry_point_matches_oracle_interact(cuda, golden):
    """Same case against the oracle's restatement of interact_beam_cpu: the
    FP64 path reproduces it to rounding."""
    e = golden("interact_cpu.npz")
    sample = ChunkedSample([(e["pos0"], e["spc0"]), (e["pos1"], e["spc1"])])
    stage = StaticStage(e["rotation"], e["translation"])
    B = _golden_beam(e)
    B._use_fast_kernel = False
    shape = tuple(int(v) for v in e["shape"])
    labels = ["Na", "Cl", "Cu"]
    ref = oracle.interact_cpu([(e["pos0"], e["spc0"]), (e["pos1"], e["spc1"])], e["coords"],
                              shape, e["rotation"], e["translation"], float(e["energy"]),
                              B.tables.f0, {l: B.tables.f0_zero(l) for l in labels},
                              B.tables.f1f2, B._beam_E0_map, B._beam_grid(),
                              B._polarization_state(), apply_polarization=True,
                              spherical_decay=True, remove_forward=True)
    got = B.interact_beam_gpu(sample, e["coords"], shape, stage, remove_forward=True,
                              apply_polarization=True, spherical_decay=True, return_double=True)
    # The stage rotates the sample: the float32 lab positions p @ R.T + t
    # round in a different order than NumPy's BLAS (1 ulp of 25 A is ~1e-5
    # rad of phase); with random atom positions that is ~4e-6 of max |A|.
    assert rel_max(got, ref) <= 1e-5, rel_max(got, ref)


def test_fcc_cu_32k_split_vs_plain(cuda):
    """The CPU-runnable configuration at full size: FP32 split-phase against
    the FP64 sum on the same GPU, and the FP64 sum against the CPU oracle on
    a pixel subset."""
    w = workloads.fcc_cu_32k()
    B = w.beam
    B._use_fast_kernel = True
    a32 = B.atomic_scattering_kinematic(w.sample, w.detector, w.stage, return_double=True, **w.sc_kwargs)
    assert B.last_run["path"] == "split_f32"
    B._use_fast_kernel = False
    a64 = B.atomic_scattering_kinematic(w.sample, w.detector, w.stage, return_double=True, **w.sc_kwargs)
    assert rel_intensity(a32, a64) <= 1e-4, rel_intensity(a32, a64)
    # The detector (7 mrad) sits inside the (111) peak of the 72 A crystal
    # (~17 mrad wide): every pixel sees the coherent sum, |A| ~ r_e N f(111).
    assert np.abs(a64).min() / 2.81794092e-15 > 0.5 * w.n_atoms * 15.0
    sel = np.s_[56:72, 56:72]
    ny, nz = w.detector.shape
    iz, iy = np.mgrid[56:72, 56:72]
    idx = (iz * ny + iy).ravel()
    pos = w.sample.load_chunk_positions(1)
    spc = w.sample.load_chunk_species(1)
    ref = oracle.interact_cpu([(pos, spc)], np.asarray(w.detector.pixel_coordinates)[:, idx],
                              (16, 16), w.stage.rotation, w.stage.translation, B._energy,
                              B.tables.f0, {"Cu": B.tables.f0_zero("Cu")}, B.tables.f1f2,
                              B._beam_E0_map, B._beam_grid(), B._polarization_state(),
                              apply_polarization=True)
    # float32 stage transform rounding (rotated sample), as above
    assert rel_max(a64[sel], ref) <= 1e-6, rel_max(a64[sel], ref)


def _single_detector(n=(6, 5), dist=5e9, tth=25.0, eta=10.0):
    D = Detector()
    D.create_detector(n, (5.5e5, 5.5e5))
    D.position_detector_absolute(dist, tth, eta)
    return D


@pytest.mark.parametrize("fast", [False, True])
def test_single_atom_known_answer(cuda, fast):
    """One atom at the origin: A = r_e (f0(Q) + f' + i f'') exp(i k r)."""
    B = Beam()
    B.create_beam(8000.0, beam_size=(100.0, 100.0))
    B._use_fast_kernel = fast
    D = _single_detector()
    S = ChunkedSample([(np.zeros((1, 3), np.float32), np.array(["Cu"]))])
    got = B.atomic_scattering_kinematic(S, D, StaticStage(), return_double=True)
    c = np.asarray(D.pixel_coordinates, np.float64) / 1e10
    r = np.linalg.norm(c, axis=0)
    Q = B.k * np.sqrt(2 * (1 - c[0] / r))
    s2 = (Q * 0.25e-10 / np.pi) ** 2
    from mosaic_gb300.tables import f0_value
    f = f0_value(B.tables.row("Cu"), s2) + B.tables.anomalous("Cu", 8000.0)
    ref = (2.81794092e-15 * f * np.exp(1j * np.fmod(B.k * r, 2 * np.pi))).reshape(D.shape[1], D.shape[0])
    assert rel_max(np.abs(got), np.abs(ref)) <= (1e-6 if fast else 1e-12)
    assert rel_max(got, ref) <= (1e-4 if fast else 1e-9)


@pytest.mark.parametrize("fast", [False, True])
def test_edge_cases(cuda, fast):
    """Ragged and degenerate inputs: tile-size remainders, a lone atom of a
    second species, atoms outside the beam grid (zero amplitude), an element
    without an f0 table (scatters nothing), a 1-pixel detector, an empty
    sample."""
    rng = np.random.default_rng(3)
    B = Beam()
    B.create_beam(10000.0, beam_size=(80.0, 80.0), beam_samples=(40, 40))
    B._use_fast_kernel = fast
    pos = (rng.random((1033, 3)) * 60 - 30).astype(np.float32)
    spc = np.array(["Si"] * 1032 + ["Au"])
    far = np.array([[0.0, 500.0, 0.0], [0.0, 0.0, -700.0]], np.float32)   # off the beam grid
    unk = np.array([[1.0, 2.0, 3.0]], np.float32)
    chunks = [(pos, spc), (far, np.array(["Si", "Si"])), (unk, np.array(["Xx"]))]
    D = _single_detector((7, 9), 2e9, 35.0, -20.0)
    got = B.atomic_scattering_kinematic(ChunkedSample(chunks), D, StaticStage(), return_double=True,
                                        apply_polarization=True, spherical_decay=True)
    ref = oracle.interact_cpu([(pos, spc)], D.pixel_coordinates, D.shape, np.eye(3), np.zeros(3),
                              10000.0, B.tables.f0, {e: B.tables.f0_zero(e) for e in ("Si", "Au")},
                              B.tables.f1f2, B._beam_E0_map, B._beam_grid(), B._polarization_state(),
                              apply_polarization=True, spherical_decay=True)
    assert rel_intensity(got, ref) <= (1e-4 if fast else 1e-10)
    # 1 pixel
    D1 = _single_detector((1, 1), 2e9, 35.0, 0.0)
    g1 = B.atomic_scattering_kinematic(ChunkedSample([(pos, spc)]), D1, StaticStage(),
                                       return_double=True)
    r1 = oracle.interact_cpu([(pos, spc)], D1.pixel_coordinates, (1, 1), np.eye(3), np.zeros(3),
                             10000.0, B.tables.f0, {e: B.tables.f0_zero(e) for e in ("Si", "Au")},
                             B.tables.f1f2, B._beam_E0_map, B._beam_grid(), B._polarization_state())
    assert rel_max(g1, r1) <= (1e-4 if fast else 1e-10)
    # empty sample
    g0 = B.atomic_scattering_kinematic(ChunkedSample([]), D, StaticStage())
    assert g0.shape == (9, 7) and not np.any(g0)


def test_complex_incident_field(cuda):
    """A custom complex wavefield: per-atom complex amplitudes reach both kernels."""
    rng = np.random.default_rng(11)
    B = Beam()
    B.create_beam(9000.0, beam_size=(90.0, 70.0), beam_samples=(30, 20))
    wf = (rng.standard_normal((30, 20)) + 1j * rng.standard_normal((30, 20))).astype(np.complex64)
    B.set_wavefield(wf)
    pos = (rng.random((3000, 3)) * 50 - 25).astype(np.float32)
    spc = rng.choice(np.array(["Fe", "O"]), 3000)
    D = _single_detector((10, 8), 3e9, 40.0, 30.0)
    outs = []
    for fast in (False, True):
        B._use_fast_kernel = fast
        outs.append(B.atomic_scattering_kinematic(ChunkedSample([(pos, spc)]), D, StaticStage(),
                                                  return_double=True, remove_forward=True))
    assert rel_intensity(outs[1], outs[0]) <= 1e-4


@pytest.mark.slow
def test_nacl_8m_linearity_full_size(cuda):
    """Full-size precision configuration: the field of the whole sample equals
    the sum of the fields of its two halves (chunks 1-8 and 9-16), each
    tiled and Morton-ordered on its own."""
    w = workloads.nacl_screw_8m()
    B = w.beam
    kw = w.sc_kwargs
    full = B.atomic_scattering_kinematic(w.sample, w.detector, w.stage, return_double=True, **kw)
    ch = w.sample._chunks
    halves = []
    for part in (ch[:8], ch[8:]):
        s = ChunkedSample([(p, (c, l)) for p, c, l in part])
        halves.append(B.atomic_scattering_kinematic(s, w.detector, w.stage, return_double=True, **kw))
    assert rel_max(halves[0] + halves[1], full) <= 2e-5
    I = np.abs(full) ** 2
    assert np.isfinite(I).all() and I.max() > 100 * np.median(I)
