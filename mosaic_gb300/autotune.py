"""Autotuner for the split-phase kernel's launch shape.

Candidates are (pixels per thread, threads per block, pixel mode); the
slice count is then chosen inside the library to fill whole waves of the GPU.
Pair candidates (one sin/cos shared by two neighbouring pixels) and quad
candidates (one by a 2x2 block) are only tried where the caller says the
geometry allows them (``level`` 1 and 2). Each candidate
is timed with CUDA events on a probe -- the first ``PROBE_TILES`` tiles
against every pixel, the same per-term work as the full problem -- the
three fastest again, interleaved, on a probe four times larger, and the
winner is cached per (device, detector-size bucket, tile size, kernel source
hash) in a JSON file, like the
reference's tune store (Beam.py:8871-8940, hardware.py:1048-1081).
"""
from __future__ import annotations

import hashlib
import json
import os
import threading

import torch

from . import engine

CANDIDATES = [(4, 128), (4, 256), (2, 256), (8, 128), (2, 128), (8, 64), (4, 64), (1, 256)]
PAIR_CANDIDATES = [(4, 128), (4, 256), (8, 128), (2, 256), (8, 64)]
QUAD_CANDIDATES = [(4, 128), (4, 256), (8, 128), (8, 64), (4, 64)]
DEFAULT = dict(pix_per_thread=4, threads=128, slices=0, pairs=0)
PROBE_TILES = 96
FINALISTS, ROUNDS, FINAL_SCALE = 3, 3, 4
KEEP_DEFAULT = 0.02
_mem = {}
_lock = threading.Lock()


def _cache_path():
    base = os.environ.get("MOSAIC_GB300_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "mosaic_gb300")
    return os.path.join(base, "tune.json")


def _src_hash():
    h = hashlib.sha1()
    for name in ("mk_split.cuh", "mk_sum_f32.cu", "mk_split_quad.cu", "mk_split_quad8.cu",
                 "mk_split_quad_ana.cu"):
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", name), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:12]


def _key(n_pix, tiles, level=0):
    dev = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    bucket = 1 << max(0, (int(n_pix) - 1).bit_length())
    return f"{dev}|{bucket}|{tiles.tile_atoms}|{'spq'[int(level)]}|{_src_hash()}"


def _load():
    try:
        with open(_cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store(key, val):
    with _lock:
        d = _load()
        d[key] = val
        p = _cache_path()
        try:
            os.makedirs(os.path.dirname(p), exist_ok=True)
            tmp = p + f".tmp{os.getpid()}"
            with open(tmp, "w") as fh:
                json.dump(d, fh, indent=1)
            os.replace(tmp, p)
        except OSError:
            pass


def lookup(n_pix, tiles, level=0):
    key = _key(n_pix, tiles, level)
    if key in _mem:
        return dict(_mem[key])
    d = _load().get(key)
    if d:
        _mem[key] = d
        return dict(d)
    return engine.default_launch(level)


def pick(finalists, times, level):
    """The run-off's winner: the fastest finalist, except that the untuned
    default (measured on full-size steps) stays unless a finalist beats it
    by more than KEEP_DEFAULT -- smaller gaps on the probe did not carry
    over to full problems (a 64-thread shape led the probe by 0.5 % and ran
    the 8.19M-atom step 3 % slower)."""
    best = finalists[min(range(len(times)), key=lambda i: times[i])]
    dflt = engine.default_launch(level)
    for cfg, t in zip(finalists, times):
        if cfg == dflt and t <= (1.0 + KEEP_DEFAULT) * min(times):
            return cfg
    return best


def tune(tiles, pix, phys, table, fresnel=0, amp_real=None, candidates=None, reps=3,
         fresnel_radius=0.0, level=0):
    """Time every candidate on a probe of the tiles; cache and return the winner."""
    amp_real = tiles.amp_is_real() if amp_real is None else bool(amp_real)
    level = int(level)
    probe = engine.TilesView(tiles, min(tiles.n_tiles, PROBE_TILES))
    # pairs only where their own bound holds (level 2 may come from quads
    # on a detector whose odd rows rule pairs out)
    pairs_ok = level >= 1 and engine.pair_delta(tiles, pix, phys.k) <= engine.PAIR_DELTA_MAX
    if candidates is None:
        candidates = [(p, t, 0) for p, t in CANDIDATES]
        if pairs_ok:
            candidates += [(p, t, 1) for p, t in PAIR_CANDIDATES]
        if level >= 2:
            candidates += [(p, t, 2) for p, t in QUAD_CANDIDATES]
    short = {1: engine.pair_short_radius(tiles, pix, phys.k) if pairs_ok else 0.0,
             2: engine.quad_bounds(tiles, pix, phys.k)["short_radius_m"] if level >= 2 else 0.0}
    def timed(view, cfg, n):
        run_cfg = dict(cfg, pair_short_radius_m=short.get(cfg["pairs"], 0.0))
        engine.run_split(view, pix, phys, table, launch=run_cfg, fresnel=fresnel,
                         amp_real=amp_real, fresnel_radius=fresnel_radius)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            engine.run_split(view, pix, phys, table, launch=run_cfg, fresnel=fresnel,
                             amp_real=amp_real, fresnel_radius=fresnel_radius)
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / n

    results = []
    for cand in candidates:
        pix_pt, nt = cand[0], cand[1]
        pr = int(cand[2]) if len(cand) > 2 else 0
        if pr > level or (pr == 1 and not pairs_ok):
            continue
        cfg = dict(pix_per_thread=pix_pt, threads=nt, slices=0, pairs=pr)
        try:
            results.append((timed(probe, cfg, reps), cfg))
        except Exception:   # a shape that does not fit the SM is skipped
            continue
    if not results:
        return dict(DEFAULT), []
    # Run-off: the first pass's leaders are within ~2 % of each other and the
    # short probe's noise is of that size, so the best FINALISTS are timed
    # again, interleaved over ROUNDS rounds, on a probe FINAL_SCALE times
    # larger; the smallest time wins.
    ranked = sorted(results, key=lambda r: r[0])
    finalists = [cfg for _, cfg in ranked[:FINALISTS]]
    if len(finalists) > 1:
        big = engine.TilesView(tiles, min(tiles.n_tiles, FINAL_SCALE * PROBE_TILES))
        best_t = {i: float("inf") for i in range(len(finalists))}
        for _ in range(ROUNDS):
            for i, cfg in enumerate(finalists):
                best_t[i] = min(best_t[i], timed(big, cfg, 1))
        best = pick(finalists, [best_t[i] for i in range(len(finalists))], level)
        results = results + [(best_t[i] / FINAL_SCALE, dict(cfg, runoff=True))
                             for i, cfg in enumerate(finalists)]
    else:
        best = finalists[0]
    key = _key(pix.n, tiles, level)
    _mem[key] = best
    _store(key, best)
    return dict(best), results
