"""Host-side pieces of the scan surrogate that need no GPU: the principal
component basis of the training frames."""
import numpy as np
import torch

from mosaic_gb300 import surrogate


def test_frame_basis_spans_the_frames():
    rng = np.random.default_rng(2)
    # 30 frames of 200 pixels on a 6-dimensional subspace (plus the mean)
    Z = rng.standard_normal((30, 6)) @ rng.standard_normal((6, 200))
    X = torch.tensor(Z + 3.0, dtype=torch.float32)
    basis = surrogate.FrameBasis(X, 16)
    assert basis.rank == 6
    assert np.allclose((basis.V @ basis.V.T).numpy(), np.eye(6), atol=1e-4)
    rec = basis.C @ basis.V + basis.mu
    assert float((rec - X).abs().max()) < 1e-3 * float(X.abs().max())
    # coefficients are ordered by variance
    v = basis.C.var(0).numpy()
    assert np.all(np.diff(v) <= 1e-6 * v[0])
