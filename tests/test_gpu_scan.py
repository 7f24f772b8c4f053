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
