"""Host side of the scan surrogate, on the CPU: the spline weights that
interpolate the training frames over the motor grid."""
import numpy as np

from mosaic_gb300 import surrogate


def test_spline_matrix_interpolates_cubics():
    """The not-a-knot cubic spline through grid nodes reproduces a cubic
    polynomial exactly, between the nodes and beyond the last one."""
    nodes = np.arange(0, 23, 4)                     # 0, 4, ..., 20 (position 22 extrapolated)
    W = surrogate.spline_matrix(23, nodes)
    x = np.arange(23, dtype=np.float64)
    f = lambda v: 0.3 * v ** 3 - 2.0 * v ** 2 + v - 5.0
    assert np.allclose(W @ f(nodes.astype(np.float64)), f(x), rtol=1e-10, atol=1e-8)
    assert np.allclose(surrogate.spline_matrix(5, [0, 4]) @ np.array([1.0, 3.0]), 1.0 + 0.5 * np.arange(5))
