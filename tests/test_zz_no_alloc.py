"""The allocation-free entry point mk_kin_split_f32_noalloc.

It serves callers that may not allocate device memory themselves through
this library -- an application whose memory pool owns the whole GPU and
passes in only the buffers to compute on, or a service whose device memory
is fixed when it starts. The test calls it through the C ABI and compares it
with the workspace entry point mk_kin_split_f32 on the same inputs and
launch shape, on two calls in a row (the shared scratch keeps the previous
call's contents, so the second call checks that nothing stale leaks into
the result), and on a detector whose usual slice count does not fit the
fixed scratch (the entry point then uses fewer slices). It builds its own
inputs, so it runs the same alone in a fresh process or after the rest of
the suite; it is collected last so that a failure here cannot stop a run
before the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

from mosaic_gb300 import _lib, engine, workloads
from mosaic_gb300._lib import MkLaunch, MkPixels

pytestmark = pytest.mark.gpu

# the tolerance of the FP32 path's parity tests; identical launch shapes make
# the two entry points agree far below it
TOL = 1e-4


def _inputs(device):
    w = workloads.fcc_cu_32k(cells=10, npix=48)
    B = w.beam
    phys = B.physics(**w.sc_kwargs)
    atoms = B.stage_atoms(w.sample, w.stage, device=device)
    tiles = engine.Tiles(atoms, B.k, 256, device=device)
    coords = np.asarray(w.detector.pixel_coordinates, dtype=np.float64) / 1e10
    pix = engine.Pixels(coords, *w.detector.shape, phys, device=device)
    return atoms.table, phys, tiles, pix


def test_noalloc_entry_matches_workspace_entry(cuda):
    L = _lib.load()
    table, phys, tiles, pix = _inputs(cuda)
    cfg = dict(pix_per_thread=4, threads=128, slices=3)
    # the factor per tile and pixel in both (the pixels passed below carry no
    # factor table)
    ref = engine.run_split(tiles, pix, phys, table, launch=cfg, fresnel=1, amp_real=False,
                           factor_table=False)
    engine.sync()
    ln = MkLaunch(4, 128, 3, 1, 0)
    sp = table.abi()
    scale = float(torch.abs(ref).max())
    for call in range(2):
        out = torch.full((pix.n, 2), float("nan"), dtype=torch.float64, device=cuda)
        rc = L.mk_kin_split_f32_noalloc(ctypes.byref(tiles.abi), ctypes.byref(sp),
                                        ctypes.byref(phys), ctypes.byref(pix.abi),
                                        ctypes.byref(ln), out.data_ptr(), 0,
                                        engine._stream_handle())
        _lib.check(rc)
        engine.sync()
        assert torch.isfinite(out).all(), call
        err = float(torch.abs(out - ref).max()) / scale
        assert err <= TOL, (call, err)


def test_noalloc_entry_caps_slices_to_the_scratch(cuda):
    """64 slices of a 512 x 512 detector need 256 MiB of partial fields, far
    more than the fixed 32 MiB: the entry point plans 7 slices instead (the
    most that fit beside the 256-byte counter), and its result equals the
    workspace entry point's run with those 7 slices (same plan, same
    fixed-order reduction) and agrees with the 64-slice run within the FP32
    path's tolerance."""
    L = _lib.load()
    w = workloads.fcc_cu_32k(cells=13, npix=512)
    B = w.beam
    phys = B.physics(**w.sc_kwargs)
    atoms = B.stage_atoms(w.sample, w.stage, device=cuda)
    tiles = engine.Tiles(atoms, B.k, 128, device=cuda)
    assert tiles.n_tiles >= 64
    coords = np.asarray(w.detector.pixel_coordinates, dtype=np.float64) / 1e10
    pix = engine.Pixels(coords, *w.detector.shape, phys, device=cuda)
    fit = (_lib.MK_NOALLOC_SCRATCH_BYTES - 256) // (16 * pix.n)
    assert fit == 7
    base = dict(pix_per_thread=4, threads=128, pairs=0)
    ref7 = engine.run_split(tiles, pix, phys, atoms.table, launch=dict(base, slices=7), fresnel=0,
                            factor_table=False)
    ref64 = engine.run_split(tiles, pix, phys, atoms.table, launch=dict(base, slices=64), fresnel=0,
                             factor_table=False)
    engine.sync()
    ln = MkLaunch(4, 128, 64, 0, int(tiles.amp_is_real()))
    sp = atoms.table.abi()
    scale = float(torch.abs(ref64).max())
    for call in range(2):
        out = torch.full((pix.n, 2), float("nan"), dtype=torch.float64, device=cuda)
        _lib.check(L.mk_kin_split_f32_noalloc(ctypes.byref(tiles.abi), ctypes.byref(sp),
                                              ctypes.byref(phys), ctypes.byref(pix.abi),
                                              ctypes.byref(ln), out.data_ptr(), 0,
                                              engine._stream_handle()))
        engine.sync()
        assert torch.isfinite(out).all(), call
        assert torch.equal(out, ref7), (call, float(torch.abs(out - ref7).max()) / scale)
        assert float(torch.abs(out - ref64).max()) / scale <= TOL, call


def test_noalloc_entry_rejects_oversized_detector(cuda):
    L = _lib.load()
    table, phys, tiles, pix = _inputs(cuda)
    big = MkPixels(3000, 1000, pix.abi.xyz, pix.abi.r0, pix.abi.q, pix.abi.u, pix.abi.phasor)
    ln = MkLaunch(4, 128, 0, 1, 0)
    sp = table.abi()
    rc = L.mk_kin_split_f32_noalloc(ctypes.byref(tiles.abi), ctypes.byref(sp), ctypes.byref(phys),
                                    ctypes.byref(big), ctypes.byref(ln), pix.abi.q, 0,
                                    engine._stream_handle())
    assert rc == _lib.MK_ENOMEM
    assert b"scratch" in L.mk_last_error()
