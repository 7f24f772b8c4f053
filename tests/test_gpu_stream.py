"""Streamed staging (chunks straight into device arrays, copied from their
own host arrays) and the on-disk sample format, on the GPU."""
import numpy as np
import pytest
import torch

from mosaic_gb300 import ChunkedSample, DiskSample, Detector, StaticStage, workloads, write_sample

pytestmark = pytest.mark.gpu


def _crystal():
    rng = np.random.default_rng(5)
    w = workloads.fcc_cu_32k(cells=8, npix=20)
    pos = w.sample.load_chunk_positions(1)
    spc = rng.choice(np.array(["Cu", "Ni", "Xx"]), size=pos.shape[0])   # Xx: no table, dropped
    cut = [0, 700, 700, 1500, pos.shape[0]]                             # one empty chunk
    return w, [(pos[a:b], spc[a:b]) for a, b in zip(cut[:-1], cut[1:])]


@pytest.mark.parametrize("thermal", [True, False])
def test_streamed_staging_equals_host_collection(cuda, thermal):
    """With a thermal model the chunks are fresh arrays; without one the
    stream reads the sample's stored arrays in place (no copy), which it
    leaves unchanged."""
    w, chunks = _crystal()
    B = workloads._beam(10000.0, 200.0)
    th = dict(sigma=0.08, max_displacement=1.0, seed=40) if thermal else None
    s = ChunkedSample(chunks, thermal=th)
    before = [s.load_chunk_positions(c) for c in range(1, s.chunk_total + 1)]
    pos_h, idx_h, labels_h = B.collect_atoms(s)
    for _ in range(2):      # a second call reuses the loader thread
        pos_d, idx_d, labels_d, counts = B.stream_atoms(s, cuda)
        assert labels_d == labels_h
        assert torch.equal(pos_d.cpu(), torch.as_tensor(pos_h))
        assert torch.equal(idx_d.cpu(), torch.as_tensor(idx_h.astype(np.int32)))
        assert np.array_equal(counts, np.bincount(idx_h, minlength=len(labels_h)))
        assert B.last_stream_bytes > 12 * pos_h.shape[0]
    for c, p in enumerate(before, start=1):
        assert np.array_equal(s.load_chunk_positions(c), p)


def test_disk_sample_through_the_entry_point(cuda, tmp_path):
    w, chunks = _crystal()
    write_sample(tmp_path, chunks)
    th = dict(sigma=0.08, max_displacement=1.0, seed=40)
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    D = Detector()
    D.create_detector((24, 20), (5.5e5, 5.5e5))
    D.position_detector_absolute(2.0e9, 2.0 * w.meta["theta_deg"], 0.0)
    st = StaticStage(w.stage.rotation, w.stage.translation)
    kw = dict(apply_polarization=True, return_double=True)
    a = B.atomic_scattering_kinematic(DiskSample(tmp_path, thermal=th), D, st, **kw)
    b = B.atomic_scattering_kinematic(ChunkedSample(chunks, thermal=th), D, st, **kw)
    assert np.array_equal(a, b)
    assert np.abs(a).max() > 0


def test_device_memory_exhaustion_sums_in_halves(cuda, monkeypatch):
    """Out of device memory while tiling: the atoms are summed in halves into
    the same field (the failure is raised on the host by a stand-in; no GPU
    memory is actually exhausted)."""
    from mosaic_gb300 import engine
    w, chunks = _crystal()
    B = workloads._beam(10000.0, 200.0, pol_perp_rate=1.0)
    D = Detector()
    D.create_detector((24, 20), (5.5e5, 5.5e5))
    D.position_detector_absolute(2.0e9, 2.0 * w.meta["theta_deg"], 0.0)
    st = StaticStage(w.stage.rotation, w.stage.translation)
    s = ChunkedSample(chunks)
    kw = dict(apply_polarization=True, return_double=True)
    ref = B.atomic_scattering_kinematic(s, D, st, **kw)
    n_all = sum(len(p) for p, _ in chunks)
    real_tiles = engine.Tiles

    class TightTiles(real_tiles):
        def __init__(self, atoms, *a, **k):
            if atoms.n > n_all // 3:
                raise torch.cuda.OutOfMemoryError("stand-in: tiles do not fit")
            super().__init__(atoms, *a, **k)

    monkeypatch.setattr(engine, "Tiles", TightTiles)
    got = B.atomic_scattering_kinematic(s, D, st, **kw)
    assert B.last_run.get("memory_splits") == 2 and B.last_run["path"] == "split_f32"
    I, Ir = np.abs(got) ** 2, np.abs(ref) ** 2
    assert np.abs(I - Ir).max() <= 1e-5 * Ir.max()

    class NoTiles(real_tiles):
        def __init__(self, atoms, *a, **k):
            raise torch.cuda.OutOfMemoryError("stand-in: nothing fits")

    monkeypatch.setattr(engine, "Tiles", NoTiles)
    with pytest.raises(RuntimeError, match="out of device memory"):
        B.atomic_scattering_kinematic(s, D, st, **kw)
