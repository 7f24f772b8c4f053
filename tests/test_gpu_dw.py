"""Debye-Waller factors exp(-B s^2) on the GPU against the oracle.

The reference has no such factor: its thermal motion is the explicit
displacement drawn on load (Sample.py:790-812), and the default B = 0 keeps
that behaviour. With B set per species, both kernels multiply each term's
scattering factor by exp(-B s^2), s = Q / (4 pi) in 1/A: the FP64 kernel per
term, the FP32 split kernel once per (tile, pixel) at the tile direction.

Tolerances as for the rest of the FP32 path: FP64 kernel vs the oracle 1e-12
of max |A| (bit-identical inputs), FP32 split vs the oracle 1e-4 relative
intensity max|I - I_ref| / max I_ref.
"""
import numpy as np
import pytest

import oracle
from helpers import kernel_case, oracle_case, rel_intensity, rel_max, run_case
from mosaic_gb300 import Detector, StaticStage, workloads
from mosaic_gb300.beam import beam as Beam
from mosaic_gb300.sample import ChunkedSample
from mosaic_gb300.tables import f0_value

pytestmark = pytest.mark.gpu

R_E = 2.81794092e-15


def _dw(s):
    """B per species index of a kernel case: distinct, up to 2.5 A^2."""
    return (0.45, 2.5, 1.1, 0.0, 1.7)[s % 5]


def test_kernel_cases_with_debye_waller(cuda, golden):
    """The reference's raw-kernel cases (3 geometries x 6 flag sets) with a
    different B per species: both kernels against the oracle's DW branch,
    and the factor visibly changes the field."""
    d = golden("kernel_cases.npz")
    effect = []
    for i in range(int(d["n"])):
        c = kernel_case(d, i)
        ref = oracle_case(c, dw=_dw)
        effect.append(rel_max(ref, oracle_case(c)))
        got64 = run_case(c, cuda, fast=False, dw=_dw)
        assert rel_max(got64, ref) <= 1e-12, (i, rel_max(got64, ref))
        for T in (128, 256):
            got32 = run_case(c, cuda, fast=True, tile_atoms=T, dw=_dw)
            assert rel_intensity(got32, ref) <= 1e-4, (i, T, rel_intensity(got32, ref))
            assert rel_max(got32, ref) <= 1e-4, (i, T, rel_max(got32, ref))
    # two of the three geometries scatter at angles where exp(-B s^2) moves
    # the field by 2-23 % of max |A|; the near-forward one by ~1e-5
    assert sum(e > 1e-2 for e in effect) >= 12, effect


@pytest.mark.parametrize("launch", [None, dict(pix_per_thread=8, threads=128, slices=0, pairs=2),
                                    dict(pix_per_thread=4, threads=128, slices=0, pairs=1)])
def test_two_species_crystal_with_debye_waller(cuda, launch):
    """A small rocksalt crystal (Na, Cl; screw dislocation) at its (002)
    reflection through the entry point, B_Na = 1.2 A^2, B_Cl = 0.7 A^2:
    FP32 split (one sin/cos per term, pixel quads, pixel pairs) and FP64
    against the oracle's restatement of interact_beam_cpu with the same B."""
    w = workloads.nacl_screw_8m(cells=(8, 8, 6), npix=24, chunk_grid=(2, 2))
    B = w.beam
    B._kernel_tile_atoms = 256
    dw = {"Na": 1.2, "Cl": 0.7}
    B.set_debye_waller(dw)
    kw = dict(w.sc_kwargs)
    chunks = [(w.sample.load_chunk_positions(c), w.sample.load_chunk_species(c))
              for c in range(1, w.sample.chunk_total + 1)]
    args = (chunks, w.detector.pixel_coordinates, w.detector.shape, w.stage.rotation,
            w.stage.translation, B._energy, B.tables.f0,
            {e: B.tables.f0_zero(e) for e in ("Na", "Cl")}, B.tables.f1f2, B._beam_E0_map,
            B._beam_grid(), B._polarization_state())
    okw = dict(apply_polarization=kw["apply_polarization"], spherical_decay=kw["spherical_decay"],
               remove_forward=kw["remove_forward"])
    ref = oracle.interact_cpu(*args, dw_b=dw, **okw)
    bare = oracle.interact_cpu(*args, **okw)
    # at (002), s^2 = 1/(4 d^2) = 0.0314 1/A^2: the peak intensity drops by
    # about exp(-2 B s^2), 5-7 %
    assert 0.85 < (np.abs(ref) ** 2).max() / (np.abs(bare) ** 2).max() < 0.97
    B._kernel_launch = launch
    B._use_fast_kernel = True
    got = B.atomic_scattering_kinematic(w.sample, w.detector, w.stage, return_double=True, **kw)
    assert B.last_run["path"] == "split_f32", B.last_run
    if launch is not None:
        assert B.last_run["launch"]["pairs"] == launch["pairs"], B.last_run
    assert rel_intensity(got, ref) <= 1e-4, rel_intensity(got, ref)
    B._use_fast_kernel = False
    got64 = B.atomic_scattering_kinematic(w.sample, w.detector, w.stage, return_double=True, **kw)
    # the rotated stage's float32 transform rounds in another order than
    # NumPy's BLAS (about 1e-6 of max |A|, as in the FP64 parity tests)
    assert rel_max(got64, ref) <= 1e-5, rel_max(got64, ref)


@pytest.mark.parametrize("fast", [False, True])
def test_single_atom_debye_waller_known_answer(cuda, fast):
    """One Fe atom at the origin, B = 1.8 A^2: |A| = r_e |f0(Q) + f' + i f''|
    exp(-B s^2), phase k r."""
    Bm = Beam()
    Bm.create_beam(9000.0, beam_size=(100.0, 100.0))
    Bm._use_fast_kernel = fast
    Bm.set_debye_waller({"Fe": 1.8})
    D = Detector()
    D.create_detector((6, 5), (5.5e5, 5.5e5))
    D.position_detector_absolute(4e9, 55.0, 10.0)
    S = ChunkedSample([(np.zeros((1, 3), np.float32), np.array(["Fe"]))])
    got = Bm.atomic_scattering_kinematic(S, D, StaticStage(), return_double=True)
    c = np.asarray(D.pixel_coordinates, np.float64) / 1e10
    r = np.linalg.norm(c, axis=0)
    Q = Bm.k * np.sqrt(2 * (1 - c[0] / r))
    s2 = (Q * 0.25e-10 / np.pi) ** 2
    f = f0_value(Bm.tables.row("Fe"), s2) + Bm.tables.anomalous("Fe", 9000.0)
    dwf = np.exp(-float(np.float32(1.8)) * s2)
    assert dwf.max() < 0.93          # the factor is far from 1 at 2 theta = 55 deg
    ref = (R_E * f * dwf * np.exp(1j * np.fmod(Bm.k * r, 2 * np.pi))).reshape(D.shape[1], D.shape[0])
    assert rel_max(np.abs(got), np.abs(ref)) <= (1e-6 if fast else 1e-12)
    assert rel_max(got, ref) <= (1e-4 if fast else 1e-9)
