"""The reference's own GPU kernel on this GPU, as a comparator.

``oracle/ref_build.py`` compiles the reference's general kernel
(``interaction_kernal``, Beam.py:1698-2415) from its own source, and
``oracle/ref_gpu.py`` launches it as the reference's ``interact_beam_gpu``
does. These tests (skipped where that source is absent):

* pin the harness: the reference's GPU kernel reproduces the reference's
  CPU fixtures (its own FP64 cffi kernel) to its FP32 accuracy;
* pin this library's analyser to the reference: the reference applies the
  top-hat and Darwin analyser only in this kernel (its CPU path ignores
  them), so the FP64 and FP32 kernels here are compared with it directly,
  at angles where the reference's float32 acos/cos resolve the factor,
  away from the top-hat's edge (where float32 cos of the acceptance moves
  the edge by ~1e-6 rad), within the reference kernel's own FP32 error.

Fields are compared in magnitude |A|: the reference kernel forms each
pixel's common phase exp(i k R0) from a float32 R0, whose rounding (~1e-8 m
at 0.1-1 m, i.e. hundreds of radians) makes that phase arbitrary while
leaving |A| intact.
"""
import numpy as np
import pytest

import oracle
from helpers import kernel_case, rel_max
from mosaic_gb300 import Detector, StaticStage
from mosaic_gb300.beam import beam as Beam
from mosaic_gb300.sample import ChunkedSample

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref_gpu(cuda):
    from oracle import ref_gpu
    if not ref_gpu.available():
        pytest.skip("the reference's GPU kernel source is not available here")
    return ref_gpu


def test_reference_gpu_kernel_reproduces_its_cpu_fixtures(cuda, golden, ref_gpu):
    """The 18 raw-kernel fixtures of the reference's FP64 cffi kernel
    (cases with a polarization axis the kernel's pol_perp_rate cannot
    express are skipped): the reference's FP32 GPU kernel agrees to its own
    accuracy (series or exact form chosen as the reference chooses it)."""
    d = golden("kernel_cases.npz")
    errs = []
    for i in range(int(d["n"])):
        c = kernel_case(d, i)
        rho = ref_gpu.pol_rate(c["pol"])
        if c["ap"] and rho is None:
            continue
        got, mode = ref_gpu.general(c["pos"], c["wk"], c["f0z"], c["anom"], c["amp"], c["cxyz"],
                                    c["ny"], c["nz"], c["k"], c["rf"], c["ap"],
                                    rho if rho is not None else 1.0, c["dc"], device=cuda)
        err = rel_max(np.abs(got), np.abs(c["cffi"].reshape(-1)))
        errs.append((i, mode, err))
    print("reference GPU kernel vs its CPU kernel:", errs)
    assert len(errs) >= 15
    assert max(e for _, _, e in errs) <= 2e-3, errs


def _wide_case():
    """Random atoms in a 30 A box; a 24 x 20 detector of 1.5 mm pixels at
    0.1 m, 2 theta = 40 deg, so pixel directions span ~0.35 x 0.3 rad."""
    rng = np.random.default_rng(17)
    pos = (rng.random((1500, 3)) * 30.0 - 15.0).astype(np.float32)
    spc = rng.choice(np.array(["Fe", "O"]), 1500)
    D = Detector()
    D.create_detector((24, 20), (1.5e7, 1.5e7))
    D.position_detector_absolute(1e9, 40.0, 0.0)
    return pos, spc, D


def _inputs(B, pos, spc):
    """Per-atom float32 inputs as the reference stages them."""
    f0 = np.stack([B.tables.row(e) for e in spc]).astype(np.float32)
    f0z = np.array([B.tables.f0_zero(e) for e in spc], np.float32)
    an = np.array([B.tables.anomalous(e, B._energy) for e in spc]).astype(np.complex64)
    amp = oracle.ein_bilinear(pos, B._beam_E0_map, *B._beam_grid())
    return (pos.astype(np.float64) / 1e10).astype(np.float32), f0, f0z, an, amp


@pytest.mark.parametrize("kind,accept,hw", [(1, 0.09, 0.0), (2, 0.0, 0.06), (2, 0.0, 0.2)])
def test_analyser_matches_the_reference_kernel(cuda, ref_gpu, kind, accept, hw):
    pos, spc, D = _wide_case()
    B = Beam()
    B.create_beam(9000.0, beam_size=(200.0, 200.0), pol_perp_rate=1.0)
    ny, nz = D.shape
    coords = np.asarray(D.pixel_coordinates, np.float64)
    cm = (coords.astype(np.float32) / np.float32(1e10))
    pos_m, f0, f0z, an, amp = _inputs(B, pos, spc)
    cidx = (nz // 2) * ny + ny // 2
    centre = cm[:, cidx]
    k = B.k
    kw = dict(apply_pol=True, pol_rate_value=1.0, device=cuda)
    ref0, mode = ref_gpu.general(pos_m, f0, f0z, an, amp, cm, ny, nz, k, **kw)
    refA, _ = ref_gpu.general(pos_m, f0, f0z, an, amp, cm, ny, nz, k,
                              analyser=(kind, centre, accept, hw), **kw)
    mode_name = {1: "top-hat", 2: "darwin"}[kind]
    S = ChunkedSample([(pos, spc)])
    outs = {}
    for fast in (False, True):
        B._use_fast_kernel = fast
        o0 = B.atomic_scattering_kinematic(S, D, StaticStage(), return_double=True,
                                           apply_polarization=True).reshape(-1)
        oA = B.atomic_scattering_kinematic(S, D, StaticStage(), return_double=True,
                                           apply_polarization=True, analyser_mode=mode_name,
                                           analyser_acceptance_angle_rad=accept,
                                           analyser_darwin_halfwidth_rad=hw).reshape(-1)
        outs[fast] = (o0, oA)
    # pixels whose direction sits within 1e-4 rad of the top-hat's edge are
    # left out (the reference resolves the edge with float32 cos)
    u = coords / np.linalg.norm(coords, axis=0)
    c = u[:, cidx]
    th = 2.0 * np.arcsin(0.5 * np.linalg.norm(u - c[:, None], axis=0))
    keep = np.ones(ny * nz, bool) if kind != 1 else np.abs(th - accept) > 1e-4
    assert keep.sum() > 0.9 * ny * nz
    if kind == 1:
        assert 0.2 < float((th <= accept).mean()) < 0.8      # the edge crosses the detector
    base = rel_max(np.abs(outs[False][0]), np.abs(ref0))     # the reference kernel's own error
    print(f"{mode_name} {mode}: reference FP32 kernel vs FP64 without analyser {base:.2e}")
    for fast, (o0, oA) in outs.items():
        err = float(np.abs(np.abs(oA) - np.abs(refA))[keep].max() / np.abs(refA).max())
        print(f"  {'split' if fast else 'plain'} with analyser vs reference: {err:.2e}")
        assert err <= 3.0 * base + 2e-4, (fast, err, base)
    # and the analyser does change the field
    assert rel_max(np.abs(refA), np.abs(ref0)) > 0.05


def test_reference_kernel_speed_on_the_headline_chunk(cuda, ref_gpu):
    """The reference's general GPU kernel against this library's split
    kernel on one 512,000-atom chunk of the headline rocksalt crystal and
    its whole 512 x 512 detector, both timed with CUDA events on this GPU
    (the reference's series order chosen as it chooses it). The split
    kernel must be the faster; the rates are written to the JSON file named
    by MOSAIC_REFERENCE_TIMING_OUT when set."""
    import json
    import os

    import torch

    from mosaic_gb300 import engine, workloads
    w = workloads.nacl_screw_8m()
    B = w.beam
    pos = w.sample.load_chunk_positions(1)
    spc = w.sample.load_chunk_species(1)
    R = np.asarray(w.stage.rotation, np.float32)
    T = np.asarray(w.stage.translation, np.float32)
    lab = (pos @ R.T + T).astype(np.float32)
    ny, nz = w.detector.shape
    coords = np.asarray(w.detector.pixel_coordinates, np.float64)
    cm = coords.astype(np.float32) / np.float32(1e10)
    pos_m, f0, f0z, an, amp = _inputs(B, lab, spc)
    n = pos_m.shape[0]
    terms = float(n) * ny * nz
    kw = dict(apply_pol=True, pol_rate_value=1.0, device=cuda)
    # warm-up (module load), then one timed run
    ref_gpu.general(pos_m[:4096], f0[:4096], f0z[:4096], an[:4096], amp[:4096], cm, ny, nz, B.k,
                    **kw)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    ref, mode = ref_gpu.general(pos_m, f0, f0z, an, amp, cm, ny, nz, B.k, **kw)
    e1.record()
    e1.synchronize()
    t_ref = e0.elapsed_time(e1) * 1e-3
    # this library's split kernel on the same chunk and pixels
    phys = B.physics(**w.sc_kwargs)
    table = engine.SpeciesTable.build(["Na", "Cl"], B.tables, B._energy)
    idx = np.where(spc == "Na", 0, 1).astype(np.int32)
    atoms = engine.atoms_lab(pos, idx, R, T, table, e0=B._beam_E0_map, grid=B._beam_grid(),
                             device=cuda)
    pix = engine.Pixels(coords / 1e10, ny, nz, phys, device=cuda)
    # the headline's form: 512-atom tiles, whose default launch is the 4x4
    # pixel square where the geometry admits it
    su, _ = B.split_setup(engine.Tiles(atoms, B.k, 512, device=cuda), pix, phys)
    cfg = engine.grouping_launch(engine.default_launch(su.level, 512), su.level, su.tiles, pix,
                                 B.k, su.info)
    run = lambda: engine.run_split(su.tiles, pix, phys, table, launch=cfg, fresnel=su.fresnel,
                                   fresnel_radius=su.fresnel_radius)
    run()
    torch.cuda.synchronize()
    e0.record()
    out = run()
    e1.record()
    e1.synchronize()
    t_ours = e0.elapsed_time(e1) * 1e-3
    ours = torch.view_as_complex(out).cpu().numpy()
    err = rel_max(np.abs(ours), np.abs(ref))
    rec = {"sample": f"{n} atoms (chunk 1 of nacl_screw_8m) x {ny}x{nz} pixels",
           "reference_kernel": "interaction_kernal (general kernel), series mode " + mode,
           "reference_gatom_px_s": terms / t_ref / 1e9, "ours_gatom_px_s": terms / t_ours / 1e9,
           "ours_launch": {k: cfg[k] for k in ("pix_per_thread", "threads", "pairs")},
           "speedup": t_ref / t_ours, "rel_max_abs_field_difference": err}
    print(rec)
    path = os.environ.get("MOSAIC_REFERENCE_TIMING_OUT")
    if path:
        with open(path, "w") as fh:
            json.dump(rec, fh)
    assert t_ours < t_ref, rec
    assert err <= 1e-2, rec
