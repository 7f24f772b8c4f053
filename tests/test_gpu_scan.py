"""Batched scans: every frame of one persistent launch against single
exposures of the same geometry, and graph replay against the first run."""
import numpy as np
import pytest

from mosaic_gb300 import workloads
from mosaic_gb300.scan import BatchedScan, frames_from_motors
from mosaic_gb300.sample import ChunkedSample
from mosaic_gb300.geometry import StaticStage

from helpers import rel_intensity

pytestmark = pytest.mark.gpu


def _small_scan():
    w = workloads.fcc_cu_32k(cells=10, npix=64)
    theta = np.radians(w.meta["theta_deg"])
    steps = [dict(mu=theta + np.radians(d), chi=np.radians(c))
             for c in (-0.4, 0.3) for d in (-1.0, -0.3, 0.0, 0.5, 1.2)]
    rois = [16, 32, 64, 24, 8, 64, 40, 32, 16, 64]
    frames = frames_from_motors(w.stage, w.detector, steps, rois)
    return w, frames


def test_batched_scan_matches_single_exposures(cuda):
    w, frames = _small_scan()
    B = w.beam
    scan = BatchedScan(B, w.sample, frames, **w.sc_kwargs)
    out, sums = scan.run()
    B._use_fast_kernel = False          # FP64 plain single exposures as the reference
    for f, fr in enumerate(frames):
        from mosaic_gb300 import Detector
        ref = B.interact_beam_gpu(w.sample, fr.pixels, fr.shape, StaticStage(fr.rotation, fr.translation),
                                  apply_polarization=True, spherical_decay=False,
                                  return_double=True)
        got = scan.frame_field(f)
        assert got.shape == ref.shape
        assert rel_intensity(got, ref) <= 1e-4, (f, rel_intensity(got, ref))
    sums_ref = np.array([np.sum(np.abs(scan.frame_field(f)) ** 2) for f in range(len(frames))])
    assert np.allclose(scan.sum_intensity(), sums_ref, rtol=1e-12)


def test_scan_graph_replay_is_bitwise(cuda):
    w, frames = _small_scan()
    scan = BatchedScan(w.beam, w.sample, frames, **w.sc_kwargs)
    out, sums = scan.run()
    first = out.clone()
    scan.capture()
    scan.out.zero_()
    scan.replay()
    import torch
    torch.cuda.synchronize()
    assert torch.equal(scan.out, first)


def test_scan_nd_batched_and_per_step_paths_agree(cuda):
    """scan_nD runs in one batched launch; with an analyser it runs one
    exposure per step instead (the analyser follows the pose). An analyser
    that accepts every direction (half-angle pi) must then give the batched
    sums; a narrow one must take intensity away."""
    from mosaic_gb300 import experiment
    w = workloads.fcc_cu_32k(cells=8, npix=32)
    th = w.meta["theta_deg"]
    args = (w.sample, w.beam, w.detector, w.stage, [(th - 0.4, th + 0.4)], [0.2], ["mu"])
    kw = dict(apply_polarization=True, spherical_decay=False, remove_forward=False)
    base = experiment.scan_nD(*args, adi_kwargs=dict(sc_kwargs=kw))["sum_intensity"]
    wide = experiment.scan_nD(*args, adi_kwargs=dict(sc_kwargs=dict(
        kw, analyser_mode="top-hat", analyser_acceptance_angle_rad=np.pi)))["sum_intensity"]
    assert base.shape == wide.shape == (5,)
    assert np.allclose(wide, base, rtol=1e-4, atol=0), (wide, base)
    narrow = experiment.scan_nD(*args, adi_kwargs=dict(sc_kwargs=dict(
        kw, analyser_mode="top-hat", analyser_acceptance_angle_rad=2e-4)))["sum_intensity"]
    assert np.all(narrow < 0.9 * base) and np.all(narrow > 0)
