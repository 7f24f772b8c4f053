"""Sharding the kinematic path over processes (one GPU each).

The path splits two ways, as in the reference (Beam.py:6182-6404,
hardware.py:1657-1713):

* an exposure over sample chunks: each rank sums its contiguous chunk range
  into a partial field and the partial fields are added (the reference adds
  its per-GPU fields on the host in device order);
* a scan over frames: each rank computes its own frames; nothing is summed.

``split_ranges`` reproduces the reference's weighted contiguous split. The
gathers go through torch.distributed (gloo for host tensors, NCCL for device
tensors); rank 0 adds partial fields in rank order, so the result does not
depend on which rank finished first.
"""
from __future__ import annotations

import numpy as np
import torch


def split_ranges(n_items, n_parts, weights=None, first=1):
    """[start, stop) per part, contiguous, sized by ``weights`` (equal by
    default); with equal weights the leading parts take the rounding, as the
    reference's split does."""
    if n_parts < 1:
        return []
    w = np.ones(n_parts) if weights is None else np.asarray(weights, dtype=np.float64)
    w = w / (w.sum() or 1.0)
    bounds = [int(first)]
    acc = 0.0
    for k, wk in enumerate(w):
        acc += wk
        stop = first + (n_items if k == len(w) - 1 else int(acc * n_items + 0.5))
        bounds.append(max(stop, bounds[-1]))
    return [(bounds[k], bounds[k + 1]) for k in range(len(w))]


class ChunkRange:
    """A view of a chunk-API sample restricted to chunks [start, stop) (1-based)."""

    def __init__(self, sample, start, stop):
        self._s, self._start, self._stop = sample, int(start), int(stop)
        self.directory = getattr(sample, "directory", "")
        self.dimensions = getattr(sample, "dimensions", None)

    @property
    def chunk_total(self):
        return max(0, self._stop - self._start)

    def chunk_atom_count(self, cid):
        return self._s.chunk_atom_count(self._start + cid - 1)

    def load_chunk_positions(self, cid, use_gpu=False, raw=False):
        return self._s.load_chunk_positions(self._start + cid - 1, use_gpu=use_gpu, raw=raw)

    def load_chunk_species(self, cid, use_gpu=False, codes=False):
        return self._s.load_chunk_species(self._start + cid - 1, use_gpu=use_gpu, codes=codes)


def sum_fields(partial, group=None):
    """Add a partial field over the ranks of the default process group, in
    rank order, on rank 0 (others get None). ``partial``: complex array."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    t = torch.view_as_real(torch.as_tensor(np.ascontiguousarray(partial, dtype=np.complex128))).contiguous()
    parts = [torch.empty_like(t) for _ in range(world)] if rank == 0 else None
    dist.gather(t, parts, dst=0, group=group)
    if rank != 0:
        return None
    acc = parts[0].clone()
    for p in parts[1:]:
        acc += p
    return torch.view_as_complex(acc).numpy()


def sharded_exposure(beam, sample, detector, stage, compute=None, **sc_kwargs):
    """One exposure split over the ranks by chunk ranges; the summed field on
    rank 0. ``compute(beam, sub_sample, detector, stage, **kw)`` returns a
    rank's complex (Nz, Ny) partial field (default: the GPU entry point with
    ``return_double=True``)."""
    import torch.distributed as dist
    world, rank = dist.get_world_size(), dist.get_rank()
    start, stop = split_ranges(int(sample.chunk_total or 0), world)[rank]
    sub = ChunkRange(sample, start, stop)
    if compute is None:
        field = beam.atomic_scattering_kinematic(sub, detector, stage, return_double=True, **sc_kwargs)
    else:
        field = compute(beam, sub, detector, stage, **sc_kwargs)
    return sum_fields(field)


def shard_frames(n_frames, rank, world):
    """The frame indices rank ``rank`` computes (contiguous, balanced)."""
    a, b = split_ranges(n_frames, world, first=0)[rank]
    return np.arange(a, b)
