"""The autotuner on the GPU: tile size and launch shape for single
exposures (``autotune.tune``, and the entry point tuning on first use) and
for batched scans (``autotune.tune_scan``); the winners are cached, looked up
again, and the tuned runs still match the oracle (relative intensity error
<= 1e-4, the FP32 path's gate)."""
import numpy as np
import pytest

import oracle
from helpers import rel_intensity
from mosaic_gb300 import StaticStage, autotune, engine, workloads
from mosaic_gb300.sample import ChunkedSample
from mosaic_gb300.scan import BatchedScan, frames_from_motors

pytestmark = pytest.mark.gpu


@pytest.fixture
def fresh_cache(tmp_path, monkeypatch):
    monkeypatch.setenv("MOSAIC_GB300_CACHE", str(tmp_path))
    autotune._mem.clear()
    yield tmp_path
    autotune._mem.clear()


def _case():
    rng = np.random.default_rng(5)
    w = workloads.fcc_cu_32k(cells=10, npix=32)
    pos = w.sample.load_chunk_positions(1)
    spc = rng.choice(np.array(["Cu", "Ni"]), size=pos.shape[0])
    return w, pos, spc


def test_tune_picks_tile_size_and_shape_and_caches(cuda, fresh_cache):
    w, pos, spc = _case()
    B = w.beam
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    atoms = B.stage_atoms(ChunkedSample([(pos, spc)]), stage, device=cuda)
    phys = B.physics(**w.sc_kwargs)
    pix = engine.Pixels(np.asarray(w.detector.pixel_coordinates, np.float64) / 1e10,
                        *w.detector.shape, phys, device=cuda)
    setups = {}
    for T in (256, 512):
        su, _ = B.split_setup(engine.Tiles(atoms, B.k, T, device=cuda), pix, phys)
        assert su is not None
        setups[T] = su
    cands = [(4, 128, 0), (8, 128, 2), (8, 128, 3), (4, 64, 1), (16, 128, 4)]
    best, table = autotune.tune(setups, pix, phys, atoms.table, candidates=cands)
    assert best["tile_atoms"] in (256, 512)
    tried = {(c["pix_per_thread"], c["threads"], c["pairs"], c["tile_atoms"]) for _, c in table}
    assert {(p, t, m, T) for p, t, m in cands for T in (256, 512)
            if m <= setups[T].level} <= tried
    assert all(ms > 0 for ms, _ in table)
    # cached on disk and in memory; lookup returns the launch for that tile size
    assert (fresh_cache / "tune.json").exists()
    assert autotune.cached(pix.n) == best
    assert autotune.tile_atoms(pix.n) == best["tile_atoms"]
    lv = setups[best["tile_atoms"]].level
    look = autotune.lookup(pix.n, lv, "exposure", best["tile_atoms"])
    assert {k: look[k] for k in ("pix_per_thread", "threads", "pairs")} == \
        {k: best[k] for k in ("pix_per_thread", "threads", "pairs")}
    # another tile size, or a level below the winner's mode: the default
    other = 256 if best["tile_atoms"] == 512 else 512
    assert autotune.lookup(pix.n, lv, "exposure", other) == engine.default_launch(lv, other)
    assert autotune.lookup(pix.n, 0, "exposure", best["tile_atoms"]) == engine.default_launch(0) \
        or best["pairs"] == 0


def test_entry_point_tunes_on_first_use(cuda, fresh_cache):
    """With ``_autotune`` on and nothing cached, the first exposure tunes
    tile size and shape, the second finds them in the cache; both match the
    oracle."""
    w, pos, spc = _case()
    B = w.beam
    B._autotune = True
    stage = StaticStage(w.stage.rotation, w.stage.translation)
    sample = ChunkedSample([(pos, spc)])
    kw = dict(w.sc_kwargs, return_double=True)
    first = B.atomic_scattering_kinematic(sample, w.detector, stage, **kw)
    assert B.last_run["launch_source"] == "tuned", B.last_run
    assert B.last_tune and B.last_run["tile_atoms"] in autotune.TILE_SIZES
    second = B.atomic_scattering_kinematic(sample, w.detector, stage, **kw)
    assert B.last_run["launch_source"] == "cached", B.last_run
    ref = oracle.interact_cpu([(pos, spc)], w.detector.pixel_coordinates, w.detector.shape,
                              stage.rotation, stage.translation, B._energy, B.tables.f0,
                              {e: B.tables.f0_zero(e) for e in ("Cu", "Ni")}, B.tables.f1f2,
                              B._beam_E0_map, B._beam_grid(), B._polarization_state(),
                              apply_polarization=w.sc_kwargs["apply_polarization"])
    for got in (first, second):
        assert rel_intensity(got, ref) <= 1e-4, rel_intensity(got, ref)


def test_scan_tunes_on_a_probe_and_caches(cuda, fresh_cache):
    """A batched scan with nothing cached tunes on a probe of its first
    frames over tile sizes and shapes; a second scan of the same size finds
    the choice in the cache; the tuned frames match single FP64 exposures."""
    w = workloads.fcc_cu_32k(cells=10, npix=64)
    B = w.beam
    B._autotune = True
    theta = np.radians(w.meta["theta_deg"])
    steps = [dict(mu=theta + np.radians(d), chi=np.radians(c))
             for c in (-0.4, 0.3) for d in (-1.0, 0.0, 0.5)]
    frames = frames_from_motors(w.stage, w.detector, steps, [16, 64, 24, 8, 40, 32])
    scan = BatchedScan(B, w.sample, frames, **w.sc_kwargs)
    assert scan.launch_source == "tuned" and scan.tune_results
    sizes = {c["tile_atoms"] for _, c in scan.tune_results}
    assert sizes == set(autotune.TILE_SIZES), sizes
    best = autotune.cached(int(scan.frame_pixels.sum()), "scan")
    assert best and best["tile_atoms"] == scan.tiles.tile_atoms
    again = BatchedScan(B, w.sample, frames, **w.sc_kwargs)
    assert again.launch_source == "cached" and again.cfg["pairs"] == scan.cfg["pairs"]
    scan.run()
    B._use_fast_kernel = False
    for f in (0, 1, 5):
        fr = frames[f]
        ref = B.interact_beam_gpu(w.sample, fr.pixels, fr.shape,
                                  StaticStage(fr.rotation, fr.translation), apply_polarization=True,
                                  spherical_decay=False, return_double=True)
        assert rel_intensity(scan.frame_field(f), ref) <= 1e-4, f
