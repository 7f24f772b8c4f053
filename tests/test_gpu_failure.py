"""Failure detection without faulting the GPU: a bounded device-side wait
that nothing satisfies expires, the kernel records the timeout and returns,
the host reads MK_ETIMEOUT, and the context keeps working."""
import numpy as np
import pytest

from mosaic_gb300 import _lib, engine
from mosaic_gb300.beam import beam as Beam
from mosaic_gb300.geometry import Detector, StaticStage
from mosaic_gb300.sample import ChunkedSample

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_context_survives(cuda):
    L = _lib.load()
    _lib.check(L.mk_debug_wait_timeout(20_000_000, engine._stream_handle()))   # 20 ms
    with pytest.raises(_lib.MosaicError) as err:
        engine.sync()
    assert err.value.code == _lib.MK_ETIMEOUT
    engine.sync()            # the status word was cleared by the read
    # the context still runs the real kernels
    B = Beam()
    B.create_beam(10000.0)
    D = Detector()
    D.create_detector((4, 4), (5.5e5, 5.5e5))
    D.position_detector_absolute(1e9, 20.0, 0.0)
    S = ChunkedSample([(np.zeros((2, 3), np.float32) + [[0, 0, 0], [1.0, 0, 0]], np.array(["C", "C"]))])
    out = B.atomic_scattering_kinematic(S, D, StaticStage())
    assert np.isfinite(out).all() and np.abs(out).max() > 0


def test_wait_probe_rejects_unbounded_limits(cuda):
    L = _lib.load()
    assert L.mk_debug_wait_timeout(0, None) == _lib.MK_EINVAL
    assert L.mk_debug_wait_timeout(5_000_000_000, None) == _lib.MK_EINVAL
