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


@pytest.mark.parametrize("ny2,nz2", [(4, 2), (8, 4), (16, 8), (32, 64), (16, 512), (8, 2048),
                                     (4, 4096), (64, 8192), (2, 8192), (1024, 1024)])
def test_fused_column_pass_matches_unfused_spectral_step(cuda, ny2, nz2):
    """mk_prop_cols between the row transforms equals the unfused step
    (2-D cuFFT, mk_prop_mul's FP64 multiply, inverse 2-D cuFFT) on random
    grids for column lengths 2..8192 (every stage-group tail, 1 to 16
    columns a block), within FP32 rounding of the transforms (relative
    2e-6 of max |A|, scaled with the transform length)."""
    from mosaic_gb300 import _lib, engine
    L = _lib.load()
    rng = np.random.default_rng(ny2 + nz2)
    P = (rng.standard_normal((nz2, ny2)) + 1j * rng.standard_normal((nz2, ny2))).astype(np.complex64)
    lam = 1.2398e-10
    k = 2 * np.pi / lam
    dy, dz, z = 2e-6, 3e-6, 0.04
    sh = engine._stream_handle()
    X = torch.as_tensor(P).to(cuda)
    F = torch.fft.fft2(X)
    _lib.check(L.mk_prop_mul(F.data_ptr(), ny2, nz2, dy, dz, k, z, k, 0.0, 0.0, sh))
    ref = torch.fft.ifft2(F, norm="forward")
    G = torch.fft.fft(X, dim=-1)
    assert G.is_contiguous()
    ws_n = int(L.mk_prop_cols_workspace_size(ny2, nz2))
    ws = torch.empty(ws_n, dtype=torch.uint8, device=cuda)
    _lib.check(L.mk_prop_cols(G.data_ptr(), ny2, nz2, dy, dz, k, z, k, 0.0, 0.0, ws.data_ptr(),
                              ws_n, sh))
    got = torch.fft.ifft(G, dim=-1, norm="forward")
    engine.sync()
    err = float((got - ref).abs().max() / ref.abs().max())
    assert err <= 2e-6 * max(1.0, np.log2(ny2 * nz2) / 8), err


def test_fused_column_pass_rejects_bad_shapes(cuda):
    from mosaic_gb300 import _lib, engine
    L = _lib.load()
    buf = torch.zeros((4, 24), dtype=torch.complex64, device=cuda)
    ws = torch.empty(4096, dtype=torch.uint8, device=cuda)
    sh = engine._stream_handle()
    k = 2 * np.pi / 1.2398e-10
    assert L.mk_prop_cols(buf.data_ptr(), 4, 24, 1e-6, 1e-6, k, 0.01, k, 0.0, 0.0, ws.data_ptr(),
                          4096, sh) == _lib.MK_EINVAL          # 24 is not a power of two
    assert L.mk_prop_cols(buf.data_ptr(), 1, 16384, 1e-6, 1e-6, k, 0.01, k, 0.0, 0.0,
                          ws.data_ptr(), 4096, sh) == _lib.MK_EINVAL   # longer than 8192
    assert L.mk_prop_cols(buf.data_ptr(), 24, 4, 1e-6, 1e-6, k, 0.01, k, 0.0, 0.0, ws.data_ptr(),
                          4096, sh) == _lib.MK_EINVAL          # rows not a power of two
    assert L.mk_prop_cols(buf.data_ptr(), 16, 4, 1e-6, 1e-6, k, 0.01, k, 0.0, 0.0, ws.data_ptr(),
                          8, sh) == _lib.MK_ENOMEM             # workspace too small


@pytest.mark.parametrize("shape,z", [((48, 40), 5e-3), ((300, 200), 0.2), ((1024, 512), 1.0)])
def test_fused_propagation_matches_unfused(cuda, shape, z):
    """The whole propagation (pad, transforms, multiply, crop) fused and
    unfused, including multi-step splits of long distances."""
    rng = np.random.default_rng(shape[0])
    ny, nz = shape
    E = (rng.standard_normal((nz, ny)) + 1j * rng.standard_normal((nz, ny))).astype(np.complex64)
    lam = 1.2398e-10
    a = propagation.propagate(E, 5.5e-5, 5.5e-5, z, lam, fused=True).cpu().numpy()
    b = propagation.propagate(E, 5.5e-5, 5.5e-5, z, lam, fused=False).cpu().numpy()
    assert np.abs(a - b).max() / np.abs(b).max() <= 5e-6
