"""The per-(species, pixel) factor table (``mk_factor_table``): its values
against a NumPy restatement of the factor at each pixel's own direction,
and the split sum with the table against the sum that evaluates the factor
per (tile, pixel), in every pixel form, and against the oracle.

Tolerances: the table's float32 arithmetic (``__expf``) against FP64 NumPy
to 2e-6 of the largest factor; the two sums to 1e-5 of max |A| (the
factor's directions differ by 2 (|o| + r) / R0 < 1e-6, far below that);
1e-4 relative intensity against the oracle (the FP32 path's gate).
"""
import numpy as np
import pytest
import torch

import oracle
from helpers import rel_intensity, rel_max
from mosaic_gb300 import Detector, StaticStage, engine, workloads
from mosaic_gb300.sample import ChunkedSample

pytestmark = pytest.mark.gpu

FORMS = {"one": dict(pix_per_thread=4, threads=128, slices=0, pairs=0),
         "quad": dict(pix_per_thread=8, threads=128, slices=0, pairs=2),
         "oct": dict(pix_per_thread=8, threads=128, slices=0, pairs=3),
         "sq": dict(pix_per_thread=16, threads=128, slices=0, pairs=4)}


def _case():
    rng = np.random.default_rng(11)
    w = workloads.fcc_cu_32k(cells=8, npix=20)
    pos = w.sample.load_chunk_positions(1)
    spc = rng.choice(np.array(["Cu", "Ni"]), size=pos.shape[0])
    return w, pos, spc


def _det(shape, theta_deg, dist=1.0e10):
    D = Detector()
    D.create_detector(shape, (5.5e5, 5.5e5))
    D.position_detector_absolute(dist, 2.0 * theta_deg, 0.0)
    return D


def _factor_numpy(table, phys, xyz_m):
    """(S, P) complex factors at the pixel directions, in FP64."""
    u = xyz_m / np.linalg.norm(xyz_m, axis=1, keepdims=True)
    b = np.asarray(phys.beam_dir[:], np.float64)
    e = np.asarray(phys.pol_e[:], np.float64)
    w = b[None, :] - u
    sf = phys.k * 0.25e-10 / np.pi
    s2 = sf * sf * (w * w).sum(1)
    out = []
    for s in range(len(table.labels)):
        wk = np.asarray(table.wk[s], np.float64)
        f0 = wk[5] + sum(wk[i] * np.exp(-wk[6 + i] * s2) for i in range(5))
        f = f0 + table.anom[s]
        if table.dw_b is not None:
            f = f * np.exp(-float(table.dw_b[s]) * s2)
        if phys.apply_pol:
            dotv, er = u @ b, u @ e
            p = 0.5 * (1 - phys.pol_deg) * (1 + dotv * dotv) + phys.pol_deg * (1 - er * er)
            f = f * np.sqrt(np.clip(p, 0.0, 1.0))
        out.append(f)
    return np.stack(out)


@pytest.mark.parametrize("dw", [False, True])
def test_factor_table_matches_numpy(cuda, dw):
    w, pos, spc = _case()
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=0.7)
    if dw:
        B.set_debye_waller({"Cu": 0.55, "Ni": 0.8})
    D = _det((24, 20), w.meta["theta_deg"])
    phys = B.physics(apply_polarization=True, spherical_decay=True)
    xyz = np.asarray(D.pixel_coordinates, np.float64) / 1e10
    pix = engine.Pixels(xyz, *D.shape, phys, device=cuda)
    table = engine.SpeciesTable.build(["Cu", "Ni"], B.tables, B._energy, B._debye_waller)
    assert (table.dw_b is not None) == dw
    got = pix.factor_table(table, phys).cpu().numpy()
    got = got[..., 0] + 1j * got[..., 1]
    want = _factor_numpy(table, phys, xyz.T)
    assert got.shape == want.shape
    scale = np.abs(want).max()
    assert np.abs(got - want).max() / scale <= 2e-6, np.abs(got - want).max() / scale
    # kept for the same table and physics, remade for another physics
    assert pix.factor_table(table, phys).data_ptr() == pix._ftab[1].data_ptr()
    phys2 = B.physics(apply_polarization=False, spherical_decay=True)
    t2 = pix.factor_table(table, phys2).cpu().numpy()
    w2 = _factor_numpy(table, phys2, xyz.T)
    assert np.abs(t2[..., 0] + 1j * t2[..., 1] - w2).max() / np.abs(w2).max() <= 2e-6


@pytest.mark.parametrize("form", sorted(FORMS))
def test_split_with_the_table_matches_the_per_tile_factor(cuda, form):
    """Cu/Ni with polarization, spherical decay and Debye-Waller factors at
    1 m: the sum with the table equals the sum that evaluates the factor per
    tile and pixel, and the oracle."""
    w, pos, spc = _case()
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=0.7)
    B.set_debye_waller({"Cu": 0.55, "Ni": 0.8})
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    D = _det((24, 20), w.meta["theta_deg"])
    phys = B.physics(apply_polarization=True, spherical_decay=True)
    atoms = B.stage_atoms(ChunkedSample([(pos, spc)]), stage, device=cuda)
    tiles = engine.Tiles(atoms, B.k, 256, device=cuda)
    pix = engine.Pixels(np.asarray(D.pixel_coordinates, np.float64) / 1e10, *D.shape, phys,
                        device=cuda)
    assert engine.factor_table_ok(tiles, pix, phys)
    level, info = engine.pixel_grouping(tiles, pix, B.k, 1e-6)
    cfg = engine.grouping_launch(FORMS[form], level, tiles, pix, B.k, info)
    assert cfg["pairs"] == FORMS[form]["pairs"], (form, level)

    def run(tab):
        o = engine.run_split(tiles, pix, phys, atoms.table, launch=cfg, fresnel=0,
                             factor_table=tab)
        engine.sync()
        a = o.cpu().numpy()
        return (a[:, 0] + 1j * a[:, 1]).reshape(D.shape[1], D.shape[0])

    with_tab, per_tile = run(True), run(False)
    assert rel_max(with_tab, per_tile) <= 1e-5, rel_max(with_tab, per_tile)
    ref = oracle.interact_cpu([(pos, spc)], D.pixel_coordinates, D.shape, stage.rotation,
                              stage.translation, B._energy, B.tables.f0,
                              {e: B.tables.f0_zero(e) for e in ("Cu", "Ni")}, B.tables.f1f2,
                              B._beam_E0_map, B._beam_grid(), B._polarization_state(),
                              apply_polarization=True, spherical_decay=True,
                              dw_b={"Cu": 0.55, "Ni": 0.8})
    assert rel_intensity(with_tab, ref) <= 1e-4, rel_intensity(with_tab, ref)


def test_entry_point_uses_the_table_where_admitted(cuda):
    """Through the entry point: the table at 1 m; not with remove_forward
    (its Q < Q_cut test stays per tile and pixel), where the split kernel
    also refuses a table it is handed."""
    w, pos, spc = _case()
    sample = ChunkedSample([(pos, spc)])
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    B._kernel_launch = FORMS["quad"]
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    D = _det((24, 20), w.meta["theta_deg"])
    B.atomic_scattering_kinematic(sample, D, stage, return_double=True, apply_polarization=True)
    assert B.last_run["path"] == "split_f32" and B.last_run["factor_table"] is True
    B.atomic_scattering_kinematic(sample, D, stage, return_double=True, apply_polarization=True,
                                  remove_forward=True)
    assert B.last_run["path"] == "split_f32" and B.last_run["factor_table"] is False
    phys = B.physics(apply_polarization=True, remove_forward=True)
    atoms = B.stage_atoms(sample, stage, device=cuda)
    tiles = engine.Tiles(atoms, B.k, 256, device=cuda)
    pix = engine.Pixels(np.asarray(D.pixel_coordinates, np.float64) / 1e10, *D.shape, phys,
                        device=cuda)
    with pytest.raises(ValueError):
        engine.run_split(tiles, pix, phys, atoms.table, launch=FORMS["one"], fresnel=0,
                         factor_table=True)


def test_scan_takes_each_frames_direction(cuda):
    """A batched scan's table holds each frame's factors (its own incident
    direction and polarization vector): every frame's slice equals a single
    exposure's table for that frame's direction."""
    from mosaic_gb300.scan import BatchedScan, frames_from_motors
    w = workloads.fcc_cu_32k(cells=6, npix=16)
    theta = np.radians(w.meta["theta_deg"])
    steps = [dict(mu=theta + np.radians(d), chi=np.radians(c)) for c in (-2.0, 3.0)
             for d in (-4.0, 5.0)]
    frames = frames_from_motors(w.stage, w.detector, steps, [16, 8, 12, 4])
    scan = BatchedScan(w.beam, w.sample, frames, launch=FORMS["quad"], **w.sc_kwargs)
    assert scan.ftab is not None
    off = 0
    for f in range(len(frames)):
        n = int(scan.frame_pixels[f])
        phys = w.beam.physics(**w.sc_kwargs)
        phys.beam_dir[:] = [float(v) for v in scan._bd[f]]
        phys.pol_e[:] = [float(v) for v in scan._pe[f]]
        xyz = scan.pix.xyz[off:off + n].t().contiguous()
        one = engine.Pixels(xyz, n, 1, phys, device=cuda)
        want = one.factor_table(scan.table, phys)
        got = scan.ftab[:, off:off + n]
        assert torch.allclose(got, want, rtol=0, atol=1e-6 * float(want.abs().max())), f
        off += n
