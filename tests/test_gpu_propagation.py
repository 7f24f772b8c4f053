"""Free-space propagation against the reference's own CPU propagator
(golden fixtures) and the FP64 oracle of the transfer-function multiply."""
import numpy as np
import pytest
import torch

import oracle
from mosaic_gb300 import Detector, propagation
from mosaic_gb300.beam import beam as Beam

pytestmark = pytest.mark.gpu


def test_prop_mul_matches_oracle(cuda, golden):
    d = golden("propagation.npz")
    k = float(d["k"])
    from mosaic_gb300 import _lib, engine
    L = _lib.load()
    for i in range(3):
        dd, z = d[f"mulcase{i}"]
        F = torch.as_tensor(d["Fs"]).to(cuda).contiguous()
        _lib.check(L.mk_prop_mul(F.data_ptr(), 24, 16, float(dd), float(dd), k, float(z), k, 0.0, 0.0,
                                 engine._stream_handle()))
        got = F.cpu().numpy()
        ref = oracle.prop_mul_f64(d["Fs"], d[f"ky{i}"].astype(np.float64) * 0 +
                                  2 * np.pi * np.fft.fftfreq(24, d=dd),
                                  2 * np.pi * np.fft.fftfreq(16, d=dd), k, z)
        scale = np.abs(d["Fs"]).max()
        assert np.abs(got - ref).max() / scale <= 1e-6, i
        # and the reference's own (float32) multiply
        assert np.abs(got - d[f"mul{i}"]).max() / scale <= 5e-5, i


def test_propagate_matches_reference_angular_spectrum(cuda, golden):
    d = golden("propagation.npz")
    lam = float(d["wavelength"])
    for i in range(2):
        dy, z = d[f"aspcase{i}"]
        got = propagation.propagate(d["field"], dy, dy, z, lam).cpu().numpy()
        ref = d[f"asp{i}"]
        assert got.shape == ref.shape
        assert np.abs(got - ref).max() / np.abs(ref).max() <= 1e-5, i


def test_wavefield_propagation_entry_point_and_fused_intensity(cuda):
    B = Beam()
    B.create_beam(10000.0)
    D = Detector()
    D.create_detector((48, 40), (1e4, 1e4))
    D.position_detector_absolute(1e10, 20.0, 0.0)
    rng = np.random.default_rng(5)
    E0 = (rng.standard_normal((40, 48)) + 1j * rng.standard_normal((40, 48))).astype(np.complex64)
    D.input_pixel_values(E0.copy())
    B.wavefield_propagation(D, propagation.FreeSpaceStack([2.0, 3.0]))
    E_two = D.pixel_values
    E_one, I = propagation.propagate(E0, 1e-6, 1e-6, 5e-3, B._wavelength, intensity=True)
    assert np.allclose(np.abs(E_one.cpu().numpy()) ** 2, I.cpu().numpy(), rtol=1e-5, atol=0)
    # two segments of 2 mm and 3 mm vs one of 5 mm: the same propagator up to
    # the crop between segments; compare away from the edges
    c = np.s_[10:30, 12:36]
    assert np.abs(E_two[c] - E_one.cpu().numpy()[c]).max() / np.abs(E0).max() <= 0.05
    with pytest.raises(ValueError):
        D.input_pixel_values(None)
        B.wavefield_propagation(D, propagation.FreeSpaceStack([1.0]))
