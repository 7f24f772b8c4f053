"""Autotuner for the split-phase kernel: atoms per tile and launch shape.

Candidates are (atoms per tile, pixels per thread, threads per block, pixel
mode); the slice count is then chosen inside the library to fill whole
waves of the GPU. Tile sizes 512, 1024 and 2048 are tried where the caller
passes the atoms (the tiles are rebuilt for each size); pair candidates
(one sin/cos shared by two neighbouring pixels) and quad candidates (one by
a 2x2 block) and octet candidates (two quads sharing their half
differences) only where that tile size's geometry allows them. Each
candidate is timed with CUDA events on a probe -- the first tiles holding
``PROBE_ATOMS`` atoms against every pixel, the same per-term work as the
full problem -- the three fastest again, interleaved, on a probe four times
larger, and the winner is cached per (device, kind of run, detector-size
bucket, kernel source hash) in a JSON file, like the reference's tune
store (Beam.py:8850-8853, 8871-8940, hardware.py:1048-1081).

Batched scans (``tune_scan``) are tuned the same way on a probe scan made of
their first frames.
"""
from __future__ import annotations

import glob
import hashlib
import json
import os
import threading
from dataclasses import dataclass, field

import torch

from . import engine

CANDIDATES = [(4, 128), (4, 256), (2, 256), (8, 128), (2, 128), (8, 64), (4, 64), (1, 256)]
PAIR_CANDIDATES = [(4, 128), (4, 256), (8, 128), (2, 256), (8, 64)]
QUAD_CANDIDATES = [(4, 128), (4, 256), (8, 128), (8, 64), (4, 64)]
OCTET_CANDIDATES = [(8, 128), (8, 256), (8, 64)]
SQUARE_CANDIDATES = [(16, 128), (16, 192)]
TILE_SIZES = (512, 1024, 2048)
DEFAULT_TILE_ATOMS = engine.DEFAULT_TILE_ATOMS
DEFAULT = dict(pix_per_thread=4, threads=128, slices=0, pairs=0)
PROBE_ATOMS = 96 * 1024
FINALISTS, ROUNDS, FINAL_SCALE = 3, 3, 4
KEEP_DEFAULT = 0.02
SCAN_PROBE_FRAMES = 8
_mem = {}
_lock = threading.Lock()


def _cache_path():
    base = os.environ.get("MOSAIC_GB300_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "mosaic_gb300")
    return os.path.join(base, "tune.json")


_SRC_HASH = []


def _src_hash():
    """Hash of every kernel source (a change to any of them retunes); taken
    once per process, as the library it describes is loaded once."""
    if _SRC_HASH:
        return _SRC_HASH[0]
    h = hashlib.sha1()
    csrc = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc")
    for path in sorted(glob.glob(os.path.join(csrc, "*.cu")) + glob.glob(os.path.join(csrc, "*.cuh"))):
        h.update(os.path.basename(path).encode())
        with open(path, "rb") as fh:
            h.update(fh.read())
    _SRC_HASH.append(h.hexdigest()[:12])
    return _SRC_HASH[0]


def _key(n_pix, kind="exposure"):
    dev = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    bucket = 1 << max(0, (int(n_pix) - 1).bit_length())
    return f"{dev}|{kind}|{bucket}|{_src_hash()}"


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


def cached(n_pix, kind="exposure"):
    """The cached winner for this device, kind and detector-size bucket (a
    launch dict with ``tile_atoms``), or None."""
    key = _key(n_pix, kind)
    if key in _mem:
        return dict(_mem[key])
    d = _load().get(key)
    if d:
        _mem[key] = d
        return dict(d)
    return None


def tile_atoms(n_pix, kind="exposure"):
    """Atoms per tile: the cached winner's, else DEFAULT_TILE_ATOMS."""
    c = cached(n_pix, kind)
    return int(c.get("tile_atoms", DEFAULT_TILE_ATOMS)) if c else DEFAULT_TILE_ATOMS


def lookup(n_pix, level=0, kind="exposure", tile_atoms=None):
    """Launch shape for a run at grouping ``level``: the cached winner when it
    was tuned for this tile size and its pixel mode is legal here, else the
    untuned default of the level."""
    c = cached(n_pix, kind)
    if c and int(c.get("pairs", 0)) <= int(level) and \
            (tile_atoms is None or int(c.get("tile_atoms", DEFAULT_TILE_ATOMS)) == int(tile_atoms)):
        c.pop("tile_atoms", None)
        return c
    return engine.default_launch(level, tile_atoms)


def pick(finalists, times, level):
    """The run-off's winner: the fastest finalist, except that the untuned
    default (measured on full-size steps) stays unless a finalist beats it
    by more than KEEP_DEFAULT -- smaller gaps on the probe did not carry
    over to full problems (a 64-thread shape led the probe by 0.5 % and ran
    the 8.19M-atom step 3 % slower)."""
    best = finalists[min(range(len(times)), key=lambda i: times[i])]
    dflt = dict(engine.default_launch(level, DEFAULT_TILE_ATOMS), tile_atoms=DEFAULT_TILE_ATOMS)
    for cfg, t in zip(finalists, times):
        c = dict(cfg)
        c.setdefault("tile_atoms", DEFAULT_TILE_ATOMS)
        if c == dflt and t <= (1.0 + KEEP_DEFAULT) * min(times):
            return cfg
    return best


@dataclass
class Setup:
    """One tile size's tiles and what its geometry allows: grouping
    ``level`` (0 none, 1 pairs, 2 quads, 3 octets, 4 squares) with ``info`` from
    engine.pixel_grouping, and whether the |d|^2 term is kept (``fresnel``)
    beyond ``fresnel_radius`` [m]."""
    tiles: object
    level: int
    info: dict = field(default_factory=dict)
    fresnel: int = 0
    fresnel_radius: float = 0.0


def candidates_for(level, pairs_ok):
    out = [(p, t, 0) for p, t in CANDIDATES]
    if pairs_ok:
        out += [(p, t, 1) for p, t in PAIR_CANDIDATES]
    if level >= 2:
        out += [(p, t, 2) for p, t in QUAD_CANDIDATES]
    if level >= 3:
        out += [(p, t, 3) for p, t in OCTET_CANDIDATES]
    if level >= 4:
        out += [(p, t, 4) for p, t in SQUARE_CANDIDATES]
    return out


def _runoff(results, timed_big, level):
    """Time the FINALISTS best again, interleaved, and pick the winner."""
    ranked = sorted(results, key=lambda r: r[0])
    finalists = [cfg for _, cfg in ranked[:FINALISTS]]
    if len(finalists) < 2:
        return finalists[0], results
    best_t = [float("inf")] * len(finalists)
    for _ in range(ROUNDS):
        for i, cfg in enumerate(finalists):
            best_t[i] = min(best_t[i], timed_big(cfg))
    best = pick(finalists, best_t, level)
    return best, results + [(best_t[i] / FINAL_SCALE, dict(cfg, runoff=True))
                            for i, cfg in enumerate(finalists)]


def _events(fn, n):
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(n):
        fn()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / n


def tune(setups, pix, phys, table, amp_real=None, reps=3, kind="exposure", candidates=None):
    """Time every candidate of every tile size on a probe; cache and return
    (winner launch dict with ``tile_atoms``, [(ms, cfg), ...]).

    ``setups``: {atoms per tile: Setup} (one entry tunes the launch shape
    only). The probes hold the same number of atoms for every tile size.
    """
    results = []
    views = {}
    top_level = max(s.level for s in setups.values())
    for T, su in sorted(setups.items()):
        tiles = su.tiles
        if not tiles.n_tiles:
            continue
        ar = tiles.amp_is_real() if amp_real is None else bool(amp_real)
        n_probe = max(1, PROBE_ATOMS // int(T))
        views[T] = (engine.TilesView(tiles, min(tiles.n_tiles, n_probe)),
                    engine.TilesView(tiles, min(tiles.n_tiles, FINAL_SCALE * n_probe)), ar, su)
        pairs_ok = bool(su.info.get("pairs_ok", su.level >= 1))
        cands = candidates if candidates is not None else candidates_for(su.level, pairs_ok)
        for cand in cands:
            pr = int(cand[2]) if len(cand) > 2 else 0
            if pr > su.level or (pr == 1 and not pairs_ok):
                continue
            cfg = dict(pix_per_thread=int(cand[0]), threads=int(cand[1]), slices=0, pairs=pr,
                       tile_atoms=int(T))
            try:
                results.append((_time_exposure(views[T][0], views[T], pix, phys, table, cfg, reps), cfg))
            except Exception:   # a shape that does not fit the SM is skipped
                continue
    if not results:
        return dict(DEFAULT, tile_atoms=DEFAULT_TILE_ATOMS), []

    def big(cfg):
        v = views[cfg["tile_atoms"]]
        return _time_exposure(v[1], v, pix, phys, table, cfg, 1)
    best, results = _runoff(results, big, top_level)
    key = _key(pix.n, kind)
    _mem[key] = best
    _store(key, best)
    return dict(best), results


def _time_exposure(view, entry, pix, phys, table, cfg, n):
    _, _, amp_real, su = entry
    run = engine.grouping_launch({k: v for k, v in cfg.items() if k != "tile_atoms"}, su.level,
                                 su.tiles, pix, phys.k, su.info)
    return _events(lambda: engine.run_split(view, pix, phys, table, launch=run, fresnel=su.fresnel,
                                            amp_real=amp_real, fresnel_radius=su.fresnel_radius), n)


def tune_scan(scan, setups, reps=2, candidates=None):
    """Tune a BatchedScan: candidates timed on a probe scan of its first
    SCAN_PROBE_FRAMES frames (all their ROI shapes) against the first tiles
    holding PROBE_ATOMS atoms. ``setups`` as in ``tune`` for the scan's own
    atoms. Returns (winner with ``tile_atoms``, results); cached per device
    and total scan pixels."""
    probe = scan.probe(min(len(scan.frames), SCAN_PROBE_FRAMES))
    results = []
    top_level = max(s.level for s in setups.values())
    plans = {}
    for T, su in sorted(setups.items()):
        if not su.tiles.n_tiles:
            continue
        n_probe = max(1, PROBE_ATOMS // int(T))
        plans[T] = (engine.TilesView(su.tiles, min(su.tiles.n_tiles, n_probe)),
                    engine.TilesView(su.tiles, min(su.tiles.n_tiles, FINAL_SCALE * n_probe)), su)
        pairs_ok = bool(su.info.get("pairs_ok", su.level >= 1))
        cands = candidates if candidates is not None else candidates_for(su.level, pairs_ok)
        for cand in cands:
            pr = int(cand[2]) if len(cand) > 2 else 0
            if pr > su.level or (pr == 1 and not pairs_ok):
                continue
            cfg = dict(pix_per_thread=int(cand[0]), threads=int(cand[1]), slices=0, pairs=pr,
                       tile_atoms=int(T))
            try:
                results.append((_time_scan(probe, plans[T][0], su, cfg, reps), cfg))
            except Exception:
                continue
    if not results:
        return dict(DEFAULT, tile_atoms=DEFAULT_TILE_ATOMS), []

    def big(cfg):
        p = plans[cfg["tile_atoms"]]
        return _time_scan(probe, p[1], p[2], cfg, 1)
    best, results = _runoff(results, big, top_level)
    key = _key(int(scan.frame_pixels.sum()), "scan")
    _mem[key] = best
    _store(key, best)
    return dict(best), results


def _time_scan(probe, view, su, cfg, n):
    probe.replan(view, su, {k: v for k, v in cfg.items() if k != "tile_atoms"})
    return _events(probe.run, n)
