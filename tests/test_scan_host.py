"""Host-side scan logic: axis construction, motor walk, couplings, detector
axes and ROIs (the frame list the batched launch consumes)."""
import numpy as np
import pytest

from mosaic_gb300 import Detector, Stage
from mosaic_gb300.experiment import axis_values, parse_ratio, scan_frames
from mosaic_gb300.scan import roi_indices


def _det():
    D = Detector()
    D.create_detector((20, 16), (5.5e5, 5.5e5))
    D.position_detector_absolute(1e10, 30.0, 0.0)
    return D


def test_axis_values_like_reference():
    assert np.allclose(axis_values(0, 1, 0.25), [0, 0.25, 0.5, 0.75, 1.0])
    assert np.allclose(axis_values(0, 1, 0.3), [0, 0.3, 0.6, 0.9, 1.0])     # endpoint appended
    assert np.allclose(axis_values(1, 0, -0.5), [1, 0.5, 0])
    assert np.allclose(axis_values(-1, 1, 1, current=10.0, relative=True), [9, 10, 11])
    with pytest.raises(ValueError):
        axis_values(0, 1, 0)
    with pytest.raises(ValueError):
        axis_values(0, 1, -0.1)
    assert parse_ratio("2:1") == 0.5 and parse_ratio(3) == 3.0
    with pytest.raises(ValueError):
        parse_ratio("0:1")


def test_scan_frames_motor_walk_matches_direct_settings():
    D, S = _det(), Stage()
    S.set_motor_value("mu", 10.0)
    axes, shape, frames = scan_frames(D, S, [(9.5, 10.5), (-1, 1)], [0.5, 1.0], ["mu", "chi"])
    assert shape == (3, 3) and len(frames) == 9
    for k, idx in enumerate(np.ndindex(*shape)):
        ref = Stage()
        ref.set_motor_value("mu", axes[0][idx[0]])
        ref.set_motor_value("chi", axes[1][idx[1]])
        assert np.allclose(frames[k].rotation, ref.rotation, atol=1e-6)
        assert frames[k].shape == (20, 16)
    # the caller's stage and detector are untouched
    assert np.isclose(np.degrees(S.motor_value[S.motor_index("mu")]), 10.0)
    assert np.isclose(np.degrees(S.motor_value[S.motor_index("chi")]), 0.0)


def test_scan_frames_couplings_detector_axes_and_rois():
    D, S = _det(), Stage()
    axes, shape, frames = scan_frames(D, S, [(0.0, 2.0)], [1.0], ["mu"],
                                      couplings={"mu": [("two_theta", "1:2")]}, rois=8)
    assert shape == (3,)
    for k, th in enumerate(axes[0]):
        ref = _det()
        ref.position_detector_absolute(1e10, 30.0 + 2.0 * th, 0.0)
        sel, sh = roi_indices(ref.shape, 8)
        assert sh == (8, 8)
        assert np.allclose(frames[k].pixels, np.asarray(ref.pixel_coordinates)[:, sel], rtol=1e-12)
    with pytest.raises(ValueError):
        scan_frames(D, S, [(0, 1)], [1], ["nonexistent"])
    with pytest.raises(ValueError):
        scan_frames(D, S, [(0, 1)] * 4, [1] * 4, ["mu", "chi", "phi", "omega"])


def test_roi_indices_are_row_major_and_clipped():
    sel, sh = roi_indices((10, 6), 4)
    assert sh == (4, 4)
    iz, iy = np.divmod(sel, 10)
    assert iy.reshape(4, 4)[0].tolist() == [3, 4, 5, 6] and iz.reshape(4, 4)[:, 0].tolist() == [1, 2, 3, 4]
    sel, sh = roi_indices((10, 6), 64)
    assert sh == (10, 6) and np.array_equal(sel, np.arange(60))
