"""Full-size benchmark configurations as parity cases (slow): the FP32
split-phase sum against the FP64 plain sum on the same GPU, over pixels
spread across the whole detector (corners, edge midpoints and a 32 x 32
grid from edge to edge: the pixel-sharing forms drop terms that grow toward
the edges and corners) and, for the polycrystal, its central 64 x 64 pixels.

Gate: max|I - I_ref| / max I_ref <= 1e-4 over the checked pixels, I_ref the
FP64 sum."""
import numpy as np
import pytest

from mosaic_gb300 import workloads
from helpers import rel_intensity

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def _fp64_at(B, w, sel, kw):
    B._use_fast_kernel = False
    coords = np.asarray(w.detector.pixel_coordinates)[:, sel]
    return B.interact_beam_gpu(w.sample, coords, (len(sel), 1), w.stage, return_double=True,
                               **kw).reshape(-1)


def _check_spread(B, w, a32, kw, label):
    sel = workloads.spread_pixels(w.detector.shape)
    a64 = _fp64_at(B, w, sel, kw)
    got = a32.reshape(-1)[sel]
    err = rel_intensity(got, a64)
    l2 = float(np.linalg.norm(np.abs(got) ** 2 - np.abs(a64) ** 2) / np.linalg.norm(np.abs(a64) ** 2))
    print(f"{label} FP32 vs FP64 over {len(sel)} spread pixels: max {err:.3e}, L2 {l2:.3e}")
    assert len(sel) >= 1024
    assert err <= 1e-4, err
    return err


def test_nacl_screw_8m_fp32_vs_fp64_whole_detector(cuda):
    """The headline configuration (8.19M atoms, 512^2 pixels, pixels sharing
    sin/cos in 2x4 octets): FP32 over the whole detector against FP64 at
    1,029 pixels that reach its corners and edges."""
    w = workloads.nacl_screw_8m()
    B = w.beam
    kw = w.sc_kwargs
    B._use_fast_kernel = True
    a32 = B.atomic_scattering_kinematic(w.sample, w.detector, w.stage, return_double=True, **kw)
    assert B.last_run["path"] == "split_f32" and B.last_run["launch"]["pairs"] >= 2, B.last_run
    _check_spread(B, w, a32, kw, "nacl_screw_8m")
    assert np.isfinite(a32).all()


def test_cu_polycrystal_18m_fp32_vs_fp64_subset(cuda):
    """64 Voronoi grains of fcc Cu (one stacking fault each) in a 60 nm cube,
    1M-atom chunks, 1024^2 pixels at 0.5 m, 12 keV: the FP32 sum over the
    whole detector, checked against the FP64 sum on the central 64 x 64
    pixels (the error reference of the configuration)."""
    w = workloads.cu_polycrystal_18m(device=cuda)
    assert 18.0e6 < w.n_atoms < 18.8e6 and w.sample.chunk_total == 19
    B = w.beam
    kw = w.sc_kwargs
    B._use_fast_kernel = True
    a32 = B.atomic_scattering_kinematic(w.sample, w.detector, w.stage, return_double=True, **kw)
    assert B.last_run["path"] == "split_f32"
    ny, nz = w.detector.shape
    iz, iy = np.mgrid[nz // 2 - 32:nz // 2 + 32, ny // 2 - 32:ny // 2 + 32]
    sel = (iz * ny + iy).ravel()
    B._use_fast_kernel = False
    a64 = B.interact_beam_gpu(w.sample, np.asarray(w.detector.pixel_coordinates)[:, sel], (64, 64),
                              w.stage, return_double=True, spherical_decay=False, **{k: v for k, v in kw.items() if k != "spherical_decay"})
    sub = a32.reshape(-1)[sel].reshape(64, 64)
    err = rel_intensity(sub, a64)
    print("polycrystal FP32 vs FP64 (central 64^2):", err, "max I", float((np.abs(a64) ** 2).max()))
    assert err <= 1e-4
    assert np.isfinite(a32).all()
    _check_spread(B, w, a32, kw, "cu_polycrystal_18m")
