"""Depth-dependent incident field on the GPU: the transmission map, depth
window and per-atom amplitudes against the reference's own outputs (golden
fixture made by running Beam._compute_beam_column_A_map_cpu,
_compute_global_depth_bounds and _ein_bilinear_cpu), and the entry point's
use_depth_ein against the oracle."""
import numpy as np
import pytest
import torch

from mosaic_gb300 import Detector, StaticStage, engine, workloads
from mosaic_gb300.beam import beam as Beam
from mosaic_gb300.sample import ChunkedSample

import oracle
from helpers import rel_intensity, rel_max

pytestmark = pytest.mark.gpu


def test_depth_maps_and_field_match_reference(cuda, golden):
    d = golden("depth_ein.npz")
    B = Beam()
    B.create_beam(float(d["energy"]), beam_size=(60.0, 60.0), beam_samples=(61, 61))
    assert np.allclose(B._beam_grid(), d["grid"], rtol=1e-12, atol=0)
    B.set_wavefield(d["E0"])
    spc = d["spc"].astype(str)
    table = engine.SpeciesTable.build(["Au", "Fe"], B.tables, B._energy)
    idx = np.where(spc == "Au", 0, 1).astype(np.int32)
    atoms = engine.atoms_lab(d["pos"], idx, d["R"], d["T"], table, e0=B._beam_E0_map,
                             grid=B._beam_grid(), device=cuda)
    tau, phi = engine.depth_maps(atoms, B._beam_E0_map.shape, B._beam_grid(),
                                 B._wavelength * 1e10, wrap=False)
    A = torch.polar(torch.exp(-tau.double()), phi.double()).cpu().numpy()
    assert np.allclose(A, d["A"], rtol=0, atol=2e-6), np.abs(A - d["A"]).max()
    # float32 lab x; the stage transform may round one ulp apart from BLAS
    assert np.allclose(engine.depth_bounds(atoms), d["s"], rtol=0, atol=1e-5)
    tau, phi, (s0, s1) = B.apply_depth_ein(atoms)
    ein = torch.view_as_complex(atoms.amp).cpu().numpy()
    ref = d["ein"]
    assert np.allclose(ein, ref, rtol=0, atol=2e-6 * np.abs(ref).max()), np.abs(ein - ref).max()
    # the transmission is visible in the field: phases move by up to ~0.03 rad
    e0_only = oracle.ein_bilinear((d["pos"] @ d["R"].T + d["T"]).astype(np.float32), d["E0"],
                                  *d["grid"])
    assert np.abs(ein - e0_only).max() > 1e-3 * np.abs(e0_only).max()


@pytest.mark.parametrize("fast", [False, True])
def test_depth_entry_point_matches_oracle(cuda, fast):
    """An 80 x 6 x 6-cell Cu/Au slab (~290 A long) at the (111) Bragg setting:
    its own transmission moves the incident phase by a few 1e-2 rad."""
    rng = np.random.default_rng(7)
    w = workloads.fcc_cu_32k(cells=8, npix=20)
    a = w.meta["a"]
    cells = np.stack(np.meshgrid(np.arange(80), np.arange(6), np.arange(6), indexing="ij"), -1)
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    pos = ((cells.reshape(-1, 1, 3) + basis[None]) * a).reshape(-1, 3)
    pos = (pos - pos.mean(0)).astype(np.float32)
    spc = rng.choice(np.array(["Cu", "Au"]), size=pos.shape[0])
    half = pos.shape[0] // 2
    sample = ChunkedSample([(pos[:half], spc[:half]), (pos[half:], spc[half:])])
    B = workloads._beam(10000.0, 600.0, pol_perp_rate=1.0)
    D = Detector()
    D.create_detector((24, 20), (5.5e5, 5.5e5))
    D.position_detector_absolute(2.0e9, 2.0 * w.meta["theta_deg"], 0.0)
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    B._use_fast_kernel = fast
    got = B.atomic_scattering_kinematic(sample, D, stage, apply_polarization=True,
                                        use_depth_ein=True, return_double=True).reshape(-1)
    assert B.last_run["path"] == ("split_f32" if fast else "plain_f64")
    args = ([(pos[:half], spc[:half]), (pos[half:], spc[half:])], D.pixel_coordinates, D.shape,
            stage.rotation, stage.translation, B._energy, B.tables.f0,
            {e: B.tables.f0_zero(e) for e in ("Cu", "Au")}, B.tables.f1f2, B._beam_E0_map,
            B._beam_grid(), B._polarization_state())
    ref = oracle.interact_cpu(*args, apply_polarization=True, depth=True).reshape(-1)
    flat = oracle.interact_cpu(*args, apply_polarization=True).reshape(-1)
    assert rel_intensity(flat, ref) > 1.5e-3        # the depth field changes the pattern
    if fast:
        assert rel_intensity(got, ref) <= 1e-4, rel_intensity(got, ref)
    else:
        assert rel_max(got, ref) <= 1e-5, rel_max(got, ref)
