"""Sharding over processes, on CPU with gloo (world size 2): a chunk-sharded
exposure summed across ranks equals the single-process sum, and frame shards
cover every frame once. The per-rank compute is the CPU oracle."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from mosaic_gb300.sharding import ChunkRange, shard_frames, split_ranges


def test_split_ranges_like_reference():
    assert split_ranges(10, 3) == [(1, 4), (4, 8), (8, 11)]
    assert split_ranges(5, 2, weights=[3, 1]) == [(1, 5), (5, 6)]
    assert split_ranges(2, 4) == [(1, 2), (2, 2), (2, 3), (3, 3)]
    ranges = split_ranges(16, 5, first=0)
    assert ranges[0][0] == 0 and ranges[-1][1] == 16
    assert all(a <= b for a, b in ranges)
    assert np.array_equal(np.concatenate([shard_frames(23, r, 4) for r in range(4)]), np.arange(23))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _oracle_compute(beam, sub, detector, stage, **kw):
    import oracle
    chunks = [(sub.load_chunk_positions(c), sub.load_chunk_species(c))
              for c in range(1, sub.chunk_total + 1)]
    labels = ["Cu", "O"]
    return oracle.interact_cpu(chunks, detector.pixel_coordinates, detector.shape, stage.rotation,
                               stage.translation, beam._energy, beam.tables.f0,
                               {e: beam.tables.f0_zero(e) for e in labels}, beam.tables.f1f2,
                               beam._beam_E0_map, beam._beam_grid(), beam._polarization_state(),
                               n_threads=1, **kw)


def _setup():
    from mosaic_gb300 import ChunkedSample, Detector, StaticStage
    from mosaic_gb300.beam import beam as Beam
    rng = np.random.default_rng(9)
    chunks = [((rng.random((n, 3)) * 30 - 15).astype(np.float32), rng.choice(["Cu", "O"], n))
              for n in (300, 120, 250, 90, 160)]
    B = Beam()
    B.create_beam(9000.0, beam_size=(100.0, 100.0))
    D = Detector()
    D.create_detector((6, 5), (5.5e5, 5.5e5))
    D.position_detector_absolute(2e9, 25.0, 5.0)
    return ChunkedSample(chunks), B, D, StaticStage()


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from mosaic_gb300.sharding import sharded_exposure
    S, B, D, St = _setup()
    field = sharded_exposure(B, S, D, St, compute=_oracle_compute, apply_polarization=True)
    if rank == 0:
        np.save(os.path.join(out_dir, "field.npy"), field)
    else:
        assert field is None
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_exposure_equals_single_process(tmp_path):
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    got = np.load(tmp_path / "field.npy")
    S, B, D, St = _setup()
    ref = _oracle_compute(B, ChunkRange(S, 1, S.chunk_total + 1), D, St, apply_polarization=True)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
