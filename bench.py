"""Benchmark of the kinematic scattering sum on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config nacl_screw_8m]

One step = one full kinematic exposure of the workload: stage transform and
incident amplitudes, species + Hilbert tiling, per-pixel prologue, the FP32
split-phase sum and the FP64 reduction. `value` is measured with the atom
positions already resident in HBM; `e2e` goes through the public entry point
``beam.atomic_scattering_kinematic`` with host arrays (host->device copies and
the device->host read of the field inside the timed region).

The workload's data (positions + tiles, ~300 MB for 8.19M atoms) exceeds the
129 MB L2, so no flush is needed between steps.

N > 1 (torchrun): every rank runs its own replica of the workload (the path
shards into independent exposures; there is no data-path collective) and
`value` is the sum over ranks of terms / max-over-ranks time ("weak" scaling).

Besides the timed steps, rank 0 reports (outside the timed region): the FP64
plain kernel on 1,029 pixels spread over the whole detector (speed and error
reference), the batched scan (all 724 frames of the 4M-atom rocking scan in
one graph-captured launch), the surrogate-assisted 101 x 101 theta x chi scan
(frames/s against the exact batched scan of all 10,201 frames, which is run
and timed too, and every returned frame's error against it) and the CPU
baseline.

--impl reference times the reference's CPU implementation on the host cores
(its own compute_scattering_cffi compiled from source into oracle/_ref, or,
where that source is absent, the oracle's C restatement of it; all threads)
on a bounded sample of the same workload, rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

PEAKS_FILE = os.path.join(HERE, "MEASURED_PEAKS.json")
MUFU_PER_CLK_SM = 16        # sin/cos results per clock per SM (MUFU)
FP32_PER_CLK_SM = 128
METRIC = "Gatom*pixel/s (kinematic sum, FP32 split-phase) vs FP64 plain on 1 GB300"
MUFU_PER_TERM, FP32_PER_TERM = 2, 12   # canonical split-phase term
# pixel-pair form: one sin/cos per two terms; per pixel pair and atom 20 FP32
# lane operations (two 3-term dot products 6, rounding 3, scale 1, delta^2 1,
# short cos/sin polynomials 3, four accumulators 4, sin/cos argument scaling
# 1, per-atom coefficients 1), run as packed f32x2 over atom pairs
MUFU_PER_TERM_PAIR, FP32_PER_TERM_PAIR = 1, 10
# 2x2 pixel-quad form: one sin/cos per four terms; per quad and atom 36 FP32
# lane operations (three dot products 9, rounding 3, scale 1, u^2 and v^2 2,
# short cos/sin polynomials of u and v 6, the four products with the phasor 4,
# eight accumulators 8, sin/cos argument scaling 1, per-atom coefficients 2)
MUFU_PER_TERM_QUAD, FP32_PER_TERM_QUAD = 0.5, 9
# 2x4 pixel-octet form (two quads sharing their half differences): per octet
# and atom 43 FP32 lane operations on tiles that pass the phase straight to
# the sin/cos (three dot products 9, the two quad phases 2, the four sin/cos
# argument scalings 2, u^2 and v^2 2, short polynomials 6, the four products
# of the shared u and v factors 4, 2 x 8 accumulators 16, per-atom
# coefficients 2) and 47 with the mod-1 reduction (4 more); ~87 % of the
# headline's tiles take the first: 5.44 per term, counted as 5.4 (the lower
# count gives the higher peak), 0.5 MUFU
MUFU_PER_TERM_OCT, FP32_PER_TERM_OCT = 0.5, 5.4
# 4x4 pixel-square form (four quads sharing their half differences): per
# square and atom 65 FP32 lane operations on tiles that pass the phase
# straight to the sin/cos (three dot products 9, the four quad phases 6, the
# four sin/cos argument scalings 4, u^2 and v^2 2, short polynomials 6, the
# four products of the shared u and v factors 4, 4 x 8 accumulators 32,
# per-atom coefficients 2) and 69 with the mod-1 reduction: 4.06-4.31 per
# term, counted as 4.0 (the lower count gives the higher peak), 0.5 MUFU
MUFU_PER_TERM_SQ, FP32_PER_TERM_SQ = 0.5, 4.0
FORMS = {0: ("one sin/cos per term", MUFU_PER_TERM, FP32_PER_TERM),
         1: ("pixel pairs (one sin/cos per two terms)", MUFU_PER_TERM_PAIR, FP32_PER_TERM_PAIR),
         2: ("2x2 pixel quads (one sin/cos per four terms)", MUFU_PER_TERM_QUAD, FP32_PER_TERM_QUAD),
         3: ("2x4 pixel octets (two quads sharing their half differences; one sin/cos per four "
             "terms)", MUFU_PER_TERM_OCT, FP32_PER_TERM_OCT),
         4: ("4x4 pixel squares (four quads sharing their half differences; one sin/cos per "
             "four terms)", MUFU_PER_TERM_SQ, FP32_PER_TERM_SQ)}


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            # the first sample takes nvidia-smi's start-up: wait for it (at most
            # 3 s) so that a short timed region still has samples around it
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            n0, t0 = len(self.lines), time.time()
            while len(self.lines) == n0 and time.time() - t0 < 0.5 and self.proc.poll() is None:
                time.sleep(0.01)             # one sample at the region's end
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _peaks():
    try:
        with open(PEAKS_FILE) as fh:
            return json.load(fh), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


TRAFFIC_PROFILES = os.path.join(HERE, "profiles")


def split_src_hash():
    """Hash of the sources the split kernel's launch is built from (its
    template and instances, its host side, the tile build and the shared
    header): the DRAM traffic of a launch depends on these alone."""
    import glob
    import hashlib
    csrc = os.path.join(HERE, "mosaic_gb300", "csrc")
    names = sorted(glob.glob(os.path.join(csrc, "mk_split*.cu")) +
                   [os.path.join(csrc, n) for n in ("mk_split.cuh", "mk_sum_f32.cu",
                                                    "mk_stage.cu", "mk_common.cuh")])
    h = hashlib.sha1()
    for path in names:
        h.update(os.path.basename(path).encode())
        with open(path, "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:12]


def profiled_traffic(config, n_pix, launch):
    """DRAM bytes per launch of the split kernel from a committed ncu
    summary of this workload (profiles/traffic_<config>.md, a line
    ``dram_bytes_per_launch: N`` with the launch shape and the split
    kernel's source hash (``split_src_hash``) it was measured on), or None. Flagged when the kernel source or
    the launch shape has changed since."""
    path = os.path.join(TRAFFIC_PROFILES, f"traffic_{config}.md")
    try:
        with open(path) as fh:
            text = fh.read()
    except OSError:
        return None
    vals = {}
    for ln in text.splitlines():
        ln = ln.strip().lstrip("-* ").strip("`")
        if ":" in ln:
            k, v = ln.split(":", 1)
            vals[k.strip()] = v.strip().strip("`")
    try:
        nbytes = int(vals["dram_bytes_per_launch"])
    except (KeyError, ValueError):
        return None
    shape = ",".join(str(launch.get(k)) for k in ("pix_per_thread", "threads", "pairs"))
    return {"bytes_per_launch": nbytes, "file": os.path.relpath(path, HERE),
            "pixels": n_pix, "measured_launch": vals.get("launch"),
            "measured_src_hash": vals.get("src_hash"),
            "same_kernel_source": vals.get("src_hash") == split_src_hash(),
            "same_launch_shape": vals.get("launch") == shape,
            "how": vals.get("how")}


def _central_subset(det_shape, m):
    ny, nz = det_shape
    iy0, iz0 = (ny - m) // 2, (nz - m) // 2
    iy, iz = np.meshgrid(np.arange(iy0, iy0 + m), np.arange(iz0, iz0 + m))
    return (iz * ny + iy).ravel()


def cpu_baseline(w, chunks=4, m=32, threads=None, reps=1):
    """The reference CPU path on host cores: ``chunks`` sample chunks x a
    central m x m pixel subset, all threads. It runs the reference's own
    kernel (compute_scattering_cffi, compiled from its source into
    oracle/_ref by oracle/ref_build.py) where that is built, else the
    oracle's FP64 C restatement of it."""
    import oracle
    B = w.beam
    threads = threads or os.cpu_count() or 1
    kernel = "reference" if oracle.ref_lib() is not None else "oracle"
    sel = _central_subset(w.detector.shape, m)
    coords = np.asarray(w.detector.pixel_coordinates)[:, sel]
    ch = []
    for cid in range(1, min(chunks, w.sample.chunk_total) + 1):
        ch.append((w.sample.load_chunk_positions(cid), w.sample.load_chunk_species(cid)))
    n_atoms = sum(c[0].shape[0] for c in ch)
    labels = sorted({str(x) for c in ch for x in np.unique(c[1])})
    f0z = {e: B.tables.f0_zero(e) for e in labels}
    args = (ch, coords, (m, m), w.stage.rotation, w.stage.translation, B._energy, B.tables.f0,
            f0z, B.tables.f1f2, B._beam_E0_map, B._beam_grid(), B._polarization_state())
    kw = dict(apply_polarization=w.sc_kwargs.get("apply_polarization", False),
              spherical_decay=w.sc_kwargs.get("spherical_decay", False),
              remove_forward=w.sc_kwargs.get("remove_forward", False), n_threads=threads,
              kernel=kernel)
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        oracle.interact_cpu(*args, **kw)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    terms = float(n_atoms) * m * m
    what = ("the reference's own compute_scattering_cffi (compiled from its source, gcc -O3), "
            "atom slices on a thread pool summed in order as interact_beam_cpu does"
            if kernel == "reference" else "FP64 C restatement of the reference CPU kernel")
    return {"value": terms / best / 1e9, "unit": "Gatom*pixel/s", "cores": int(threads),
            "kind": "reference" if kernel == "reference" else "port",
            "sample": f"{n_atoms} atoms ({len(ch)} of {w.sample.chunk_total} chunks) x central "
                      f"{m}x{m} pixels, {what}, {threads} threads, {best:.2f} s"}


def probe_pipes(dev):
    """Per-clock per-SM throughput of the MUFU (sin+cos), FRND and FFMA pipes
    on this GPU (mk_probe_throughput)."""
    import ctypes

    import torch

    from mosaic_gb300 import _lib, engine
    L = _lib.load()
    ws_n = int(L.mk_probe_workspace_size())
    ws = torch.empty(ws_n, dtype=torch.uint8, device=dev)
    out = {}
    for kind, name, iters in ((1, "sincos", 2048), (2, "frnd", 2048), (3, "ffma", 16384)):
        v = ctypes.c_double(0.0)
        _lib.check(L.mk_probe_throughput(kind, iters, ws.data_ptr(), ws_n, ctypes.byref(v),
                                         engine._stream_handle()))
        out[name] = float(v.value)
    return out


def scan_leg(args, dev):
    """Batched scan: the 724 frames of the 4M-atom rocking x chi scan (181
    theta steps x 4 chi offsets, ROI sides cycling 64/128/256/512), all in
    one persistent launch captured in a CUDA graph; frames/s of one replay.
    The scan's tile size and launch shape come from the autotuner (tuned on
    a probe of the first frames when not cached); the kernels are warmed on
    an 8-frame scan of the same staged atoms, so the whole scan runs once,
    timed."""
    import torch

    from mosaic_gb300 import workloads
    from mosaic_gb300.scan import BatchedScan, frames_from_motors

    w = workloads.cu_bumps_scan_4m()
    fr = w.meta["frames"][: args.scan_frames]
    frames = frames_from_motors(w.stage, w.detector, [dict(mu=f["mu"], chi=f["chi"]) for f in fr],
                                [f["roi"] for f in fr])
    t0 = time.perf_counter()
    scan = BatchedScan(w.beam, w.sample, frames, **w.sc_kwargs)   # tuned on a probe if not cached
    setup_s = time.perf_counter() - t0
    scan.probe(8, launch=scan.cfg).run()                           # first use of the launch shape
    torch.cuda.synchronize()
    scan.capture(warm=False)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(int(dev.index or 0)) as sampler:
        e0.record()
        scan.replay()
        e1.record()
        e1.synchronize()
    s = e0.elapsed_time(e1) * 1e-3
    npx = int(scan.frame_pixels.sum())
    return {"workload": "cu_bumps_scan_4m", "frames": len(frames), "frames_total_in_config": 724,
            "atoms": scan.atoms.n, "pixels": npx, "terms": scan.terms,
            "frames_per_s": len(frames) / s, "terms_per_s": scan.terms / s, "seconds": s,
            "setup_seconds": setup_s, "graph": True, "launch": dict(scan.cfg),
            "launch_source": scan.launch_source, "tile_atoms": scan.tiles.tile_atoms,
            "autotune": [[float(t), c] for t, c in scan.tune_results], "clocks": sampler.summary(),
            "note": "the 181 theta x 4 chi rocking scan; ROI sides 64/128/256/512 by frame index; "
                    "atoms staged once, all frames one persistent launch, one timed graph replay"}


def surrogate_leg(args, dev):
    """Surrogate-assisted scan on the 101 x 101 theta x chi grid (+-0.3 deg)
    of the 4M-atom crystal, 128^2 ROI: training frames every 4th point per
    axis, every 8th predicted frame judged exactly, 2% fallback. With
    ``--surrogate-exact-all`` the exact-only scan of all 10,201 frames is run
    and timed too (and every returned frame checked against it); otherwise
    its time is the exact launch's per-frame time (same batched kernel) times
    the 10,201 frames."""
    import torch

    from mosaic_gb300 import workloads
    from mosaic_gb300.surrogate import SurrogateScan

    w = workloads.cu_bumps_surrogate_4m()
    m = w.meta
    sc = SurrogateScan(w.beam, w.sample, w.detector, w.stage, m["theta_offsets"], m["chi_offsets"],
                       roi=m["roi"], stride=4, judge_every=8, tol=0.02, sc_kwargs=w.sc_kwargs)
    res = sc.run(verify=args.surrogate_verify, exact_all=args.surrogate_exact_all)
    torch.cuda.synchronize()
    ve = res.get("verify_err", np.zeros(0))
    if args.surrogate_exact_all:
        # every frame computed exactly (that pass is the measured exact-only
        # scan): the error of every frame the surrogate returned
        ve = np.asarray(res["final_err"])
    pct = lambda x: [float(np.percentile(x, q)) for q in (50, 90, 99, 100)] if len(x) else None
    return {"workload": "cu_bumps_surrogate_4m", "grid": m["grid"], "roi": m["roi"],
            "reading": "training frames every 4th point per axis (26 x 26)",
            "frames": res["n_frames"], "frames_per_s": res["frames_per_s"],
            "exact_frames_per_s": res["exact_frames_per_s"], "gain": res["gain"],
            "exact_seconds": res["exact_seconds"], "exact_measured": bool(res["exact_measured"]),
            "seconds": res["seconds"], "exact_frames": res["exact_frames"],
            "n_train": res["n_train"], "n_judged": res["n_judged"],
            "n_failed_judges": res["n_failed_judges"], "n_fallback": res["n_fallback"],
            "times": res["times"],
            "judge_err_p50_p90_p99_max": pct(res["judge_err"]),
            "judge_err_spline_only_p50_p90_p99_max": pct(res["judge_err_base"]),
            "checked_err_p50_p90_p99_max": pct(ve), "checked": int(len(ve)),
            "checked_frac_within_tol": float((ve <= 0.02).mean()) if len(ve) else None,
            "all_frames": ({"n": int(len(res["final_err"])),
                            "max_err": float(np.max(res["final_err"])),
                            "frac_within_tol": float((np.asarray(res["final_err"]) <= 0.02).mean()),
                            "prediction_err_p50_p90_p99_max": pct(np.asarray(res["model_err"])),
                            "spline_only_err_p50_p90_p99_max": pct(np.asarray(res["base_err"]))}
                           if "final_err" in res else None),
            "mlp": {"networks": 2, "params_each": res["params"], "components": res["rank"],
                    "final_loss": res["final_loss"],
                    "dtype": "bf16 weights/activations, fp32 accumulate",
                    "training": _mlp_rate(2 * res["params"],
                                          res["n_train"] + res["n_judged"] / 2.0, sc.fit_steps,
                                          res["times"]["fit"])}}


def _mlp_rate(params, n_train, steps, seconds):
    """The surrogate's training against the bf16 tensor peak: 6 flops per
    parameter and sample a step (forward 2, backward 4), over the fit phase
    (which also holds the frame basis and target set-up)."""
    peaks, src = _peaks()
    flops = 6.0 * float(params) * float(n_train) * float(steps)
    tf = flops / max(seconds, 1e-12) / 1e12
    peak = float(peaks.get("bf16_tflops", 1900.0))
    return {"flops": flops, "tflops": tf, "peak_tflops": peak, "frac": tf / peak,
            "peak_source": src,
            "note": "latency-bound by design: the layers are 676 x 256 x 256 GEMMs "
                    "(~0.1 GFLOP, a few microseconds each), far too small to fill "
                    "the tensor cores; the whole fit is ~2 % of the scan's time"}


def fp64_spread_check(w, field, dev, n_grid=32):
    """The FP64 plain GPU kernel on pixels spread over the whole detector
    (the 4 corners, the 4 edge midpoints, the centre and an n_grid x n_grid
    edge-to-edge grid) of workload ``w``, all atoms: its rate (the speed
    bar) and the errors of ``field`` (complex (nz, ny), the FP32 split
    result) against it. The pixel-sharing forms drop terms that grow toward
    the detector's edges and corners, so the error is taken there too."""
    import torch

    from mosaic_gb300 import engine, workloads
    B = w.beam
    kw = w.sc_kwargs
    phys = B.physics(kw["apply_polarization"], kw["spherical_decay"], kw["remove_forward"])
    pos_h, idx_h, labels = B.collect_atoms(w.sample)
    table = engine.SpeciesTable.build(labels, B.tables, B._energy, B._debye_waller)
    coords_m = np.asarray(w.detector.pixel_coordinates, dtype=np.float64) / 1e10
    ny, nz = w.detector.shape
    sel = workloads.spread_pixels(w.detector.shape, n_grid)
    m = len(sel)
    pix_s = engine.Pixels(coords_m[:, sel], m, 1, phys, device=dev)
    a = engine.atoms_lab(torch.as_tensor(pos_h).to(dev), idx_h, w.stage.rotation,
                         w.stage.translation, table, e0=B._beam_E0_map, grid=B._beam_grid(),
                         device=dev)
    torch.cuda.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record()
    ref = engine.run_plain(a, pix_s, phys)
    f1.record()
    engine.sync()
    fp64_s = f0.elapsed_time(f1) * 1e-3
    I_ref = (ref ** 2).sum(1).cpu().numpy()
    I_out = np.abs(np.asarray(field).reshape(-1)[sel]) ** 2
    strong = I_ref >= 1e-3 * I_ref.max()
    edge = np.isin(sel, workloads.spread_pixels(w.detector.shape, 2)) & \
        (sel != (nz // 2) * ny + ny // 2)
    return {"fp64_gatom_px_s": float(pos_h.shape[0]) * m / fp64_s / 1e9, "pixels": m,
            "rel_err_max_over_peak": float(np.abs(I_out - I_ref).max() / I_ref.max()),
            "rel_err_l2": float(np.linalg.norm(I_out - I_ref) / np.linalg.norm(I_ref)),
            "rel_err_corners_and_edge_midpoints": float(np.abs(I_out - I_ref)[edge].max()
                                                        / I_ref.max()),
            "rel_err_local_max_where_I_ge_1e-3_peak":
                float((np.abs(I_out - I_ref)[strong] / I_ref[strong]).max()) if strong.any()
                else None}


def configs_leg(args, dev, reps=3):
    """The other single-exposure configurations -- config 1 (32,000-atom fcc
    Cu, 128^2) and config 3 (18.3M-atom Cu polycrystal, 1024^2) -- end to end
    through the public entry point with host arrays (median of ``reps``
    calls after one call that stages, and tunes on first use of the detector
    size), each checked against the FP64 plain kernel on pixels spread over
    its whole detector."""
    import torch

    from mosaic_gb300 import workloads
    out = {}
    for name in ("fcc_cu_32k", "cu_polycrystal_18m"):
        w = workloads.build(name)
        B = w.beam
        kw = w.sc_kwargs
        B.atomic_scattering_kinematic(w.sample, w.detector, w.stage, return_double=True, **kw)
        times = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            field = B.atomic_scattering_kinematic(w.sample, w.detector, w.stage,
                                                  return_double=True, **kw)
            times.append(time.perf_counter() - t0)
        s = float(np.median(times))
        n_atoms = int(B.collect_atoms(w.sample)[0].shape[0])
        n_pix = int(np.prod(w.detector.shape))
        terms = float(n_atoms) * n_pix
        chk = fp64_spread_check(w, field, dev, args.fp64_grid)
        out[name] = {"atoms": n_atoms, "pixels": n_pix, "e2e_seconds": s,
                     "e2e_gatom_px_s": terms / s / 1e9,
                     "speedup_vs_fp64": terms / s / 1e9 / chk["fp64_gatom_px_s"],
                     "path": B.last_run.get("path"), "tile_atoms": B.last_run.get("tile_atoms"),
                     "launch": B.last_run.get("launch"),
                     "accuracy_vs_fp64": chk}
        del w, B, field
        torch.cuda.empty_cache()
    return out


def gemm_profile_case():
    """The scan surrogate's two tcgen05 GEMM shapes, each launched twice
    (warm-up, then timed with CUDA events): (a) one MLP layer for the group
    of two networks, 2 x (1,272 x 256 x 256), bias + ReLU epilogue with FP32
    and BF16 outputs; (b) the frame decode, 8,334 x 16,384 x 192, epilogue
    adding the mean frame, clamping, scaling rows and storing them at their
    frames' rows of a 10,201-frame output. Launch order a, a, b, b (the
    kernel-profile commands select launch 1 or 3)."""
    import ctypes

    import torch

    from mosaic_gb300 import _lib, engine
    L = _lib.load()
    dev = torch.device("cuda")
    p = lambda t: t.data_ptr() if t is not None else None
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    M, N, K, G = 1272, 256, 256, 2
    A = torch.randn((G, M, K), device=dev, generator=g).bfloat16()
    W = torch.randn((G, N, K), device=dev, generator=g).bfloat16()
    b = torch.randn((G, N), device=dev, generator=g)
    C = torch.empty((G, M, N), device=dev)
    Cb = torch.empty((G, M, N), device=dev, dtype=torch.bfloat16)
    gs = (ctypes.c_longlong * 6)(M * K, N * K, M * N, M * N, N, 0)
    Md, Nd, Kd = 8334, 16384, 192
    Ad = torch.randn((Md, Kd), device=dev, generator=g).bfloat16()
    Bt = torch.randn((Nd, Kd), device=dev, generator=g).bfloat16()
    mu = torch.randn(Nd, device=dev, generator=g)
    scale = torch.rand(Md, device=dev, generator=g)
    rows = torch.randperm(10201, device=dev, generator=g)[:Md].contiguous()
    out = torch.empty((10201, Nd), device=dev)

    def run_a():
        _lib.check(L.mk_gemm_tc_groups(G, gs, M, N, K, p(A), K, 1, p(W), 1, K, p(C), N, p(b), 6,
                                       p(Cb), N, None, 0, None, None, engine._stream_handle()))

    def run_b():
        _lib.check(L.mk_gemm_tc(Md, Nd, Kd, p(Ad), Kd, 1, p(Bt), 1, Kd, p(out), Nd, p(mu), 6, None,
                                0, None, 0, p(scale), p(rows), engine._stream_handle()))

    res = {}
    for name, fn, flops, nbytes in (("mlp_layer_two_networks", run_a, 2.0 * G * M * N * K,
                                     G * M * N * 6),
                                    ("frame_decode", run_b, 2.0 * Md * Nd * Kd, Md * Nd * 4)):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        res[name] = {"us": ms * 1e3, "tflops": flops / ms / 1e9, "gb_s_written": nbytes / ms / 1e6}
    _lib.check(L.mk_sync_status(engine._stream_handle()))
    print(json.dumps({"gemm_profile": res}))


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return
    from mosaic_gb300 import workloads
    w = workloads.build(args.config)
    threads = os.cpu_count() or 1
    steps = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(w, chunks=1, m=16, threads=threads)
        if i >= args.warmup:
            steps.append(r)
    val = float(np.median([s["value"] for s in steps]))
    line = {"impl": "reference", "metric": METRIC, "value": val,
            "unit": "Gatom*pixel/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.config, "atoms": int(sum(w.sample.chunk_atom_count(c)
                                                                  for c in range(1, w.sample.chunk_total + 1))),
                       "pixels": int(np.prod(w.detector.shape)), "host_cores": threads,
                       "sample": "one chunk x central 16x16 pixels per step (terms/s is linear in atoms "
                                 "and pixels)"},
            "cpu_baseline": {"value": val, "unit": "Gatom*pixel/s", "cores": threads,
                             "kind": steps[-1]["kind"], "sample": steps[-1]["sample"]},
            "e2e": {"value": val, "unit": "Gatom*pixel/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args):
    import torch
    import torch.distributed as dist

    from mosaic_gb300 import autotune, engine, workloads

    rank, world, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    w = workloads.build(args.config)
    B = w.beam
    if args.tile_atoms:
        B._kernel_tile_atoms = int(args.tile_atoms)
    kw = w.sc_kwargs
    phys = B.physics(kw["apply_polarization"], kw["spherical_decay"], kw["remove_forward"])
    pos_h, idx_h, labels = B.collect_atoms(w.sample)
    table = engine.SpeciesTable.build(labels, B.tables, B._energy, B._debye_waller)
    pos_d = torch.as_tensor(pos_h).to(dev)             # resident inputs
    idx_d = torch.as_tensor(idx_h.astype(np.int32)).to(dev)
    counts = np.bincount(idx_h, minlength=len(labels)).astype(np.int64)
    coords_m = np.asarray(w.detector.pixel_coordinates, dtype=np.float64) / 1e10
    coords_d = torch.as_tensor(coords_m).to(dev)
    ny, nz = w.detector.shape
    n_atoms, n_pix = pos_h.shape[0], ny * nz
    terms = float(n_atoms) * n_pix

    # Tile size and launch shape: autotuned once on a probe (tile sizes 512,
    # 1024 and 2048, each with the pixel forms its geometry allows), cached
    # on disk; the entry point then finds the same choice in the cache.
    atoms = engine.atoms_lab(pos_d, idx_h, w.stage.rotation, w.stage.translation, table,
                             e0=B._beam_E0_map, grid=B._beam_grid(), device=dev)
    pix = engine.Pixels(coords_m, ny, nz, phys, device=dev)
    sizes = [int(args.tile_atoms)] if args.tile_atoms else list(autotune.TILE_SIZES)
    if args.profile and not args.tile_atoms:
        sizes = [B.tile_atoms_for(n_pix)]
    setups = {}
    for T in sizes:
        t = engine.Tiles(atoms, B.k, T, device=dev)
        su, diag_T = B.split_setup(t, pix, phys)
        if su is None:
            continue
        if args.no_pairs:
            su.level = 0
        elif args.no_quads:
            su.level = min(su.level, 1 if su.info["pairs_ok"] else 0)
        elif args.no_octets:
            su.level = min(su.level, 2)
        elif args.no_squares:
            su.level = min(su.level, 3)
        setups[T] = su
    if not setups:
        raise RuntimeError(f"{args.config}: the split form declines this geometry")
    if args.launch:
        ppt, nt, mode = (int(v) for v in args.launch.split(","))
        T = sizes[0] if len(sizes) == 1 else (512 if 512 in setups else min(setups))
        launch, tune_tbl = dict(pix_per_thread=ppt, threads=nt, slices=0, pairs=mode), []
    elif args.profile:
        T = min(setups)
        launch, tune_tbl = autotune.lookup(pix.n, setups[T].level, "exposure", T), []
    else:
        best, tune_tbl = autotune.tune(setups, pix, phys, table)
        T = int(best.pop("tile_atoms"))
        launch = best
    su = setups[T]
    del setups
    tiles, level, ginfo = su.tiles, su.level, su.info
    _, diag = B.split_setup(tiles, pix, phys)
    diag.update(ginfo)
    fresnel = su.fresnel
    B._kernel_tile_atoms = T
    launch = engine.grouping_launch(launch, level, tiles, pix, B.k, ginfo)
    B._kernel_launch = launch
    amp_real = tiles.amp_is_real()
    # the per-(species, pixel) factor table where the geometry admits it,
    # decided once (the check reads back the tile and pixel extents)
    ftab = (not args.no_factor_table) and engine.factor_table_ok(tiles, pix, phys)
    split_times = []

    def step(record=False):
        a = engine.atoms_lab(pos_d, idx_d, w.stage.rotation, w.stage.translation, table,
                             e0=B._beam_E0_map, grid=B._beam_grid(), device=dev, counts=counts)
        t = engine.Tiles(a, B.k, T, device=dev)
        p = engine.Pixels(coords_d, ny, nz, phys, device=dev)
        if record:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
        out = engine.run_split(t, p, phys, table, launch=launch, fresnel=fresnel,
                               amp_real=amp_real, fresnel_radius=su.fresnel_radius,
                               factor_table=ftab)
        if record:
            e1.record()
            split_times.append((e0, e1))
        return out

    for _ in range(args.warmup):
        step()
    barrier()
    sampler = ClockSampler(local)
    with sampler:
        barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(args.steps):
            out = step(record=True)
        ev1.record()
        barrier()
    engine.sync()
    ms = ev0.elapsed_time(ev1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    split_ms = float(np.mean([a.elapsed_time(b) for a, b in split_times]))
    value = terms * world / (ms * 1e-3) / 1e9
    clocks = sampler.summary()
    if args.profile:
        # Kernel-profile run: one configuration, no side legs.
        if rank == 0:
            print(json.dumps({"profile": args.config, "ms_per_step": ms, "split_ms": split_ms,
                              "value": value, "launch": launch, "fresnel": bool(fresnel),
                              "factor_table": bool(ftab)}))
        return

    # End to end through the public entry point with host buffers.
    # one untimed call first (the entry point's first use: its loader
    # thread, the first touch of the sample's host pages by the copy
    # engines), then the median of three calls
    B.atomic_scattering_kinematic(w.sample, w.detector, w.stage, return_double=True, **kw)
    e2e_times = []
    for i in range(max(2, min(3, args.steps))):
        barrier()
        t0 = time.perf_counter()
        field = B.atomic_scattering_kinematic(w.sample, w.detector, w.stage, return_double=True,
                                              **kw)
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = float(np.median(e2e_times))
    if world > 1:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    # what the entry point copies: the streamed chunks (positions, species
    # codes), the beam map and the pixel coordinates
    # (the pixel coordinates only when the call prepared its pixels: the
    # entry point keeps them across calls with an unchanged detector)
    h2d = int(getattr(B, "last_stream_bytes", pos_h.nbytes + 4 * n_atoms)) + \
        B._beam_E0_map.astype(np.complex64).nbytes + \
        (0 if getattr(B, "last_pixels_cached", False) else coords_m.nbytes)
    d2h = n_pix * 16

    # FP64 plain (same GPU) on pixels spread over the whole detector: speed
    # bar and error reference
    chk = fp64_spread_check(w, field, dev, args.fp64_grid)
    m, fp64_rate = chk["pixels"], chk["fp64_gatom_px_s"]

    peaks, peak_src = _peaks()
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    clk = float(peaks.get("sm_max_mhz", 2070.0))
    pipes = probe_pipes(dev)
    mufu = pipes.get("sincos", MUFU_PER_CLK_SM)
    fma = pipes.get("ffma", FP32_PER_CLK_SM)
    # canonical term (2 MUFU + 12 FP32) for the roofline, whatever form runs;
    # the running form's own bound (pixel pairs or quads) beside it
    mode = int(launch.get("pairs", 0) or 0)
    peak_terms = min(mufu / MUFU_PER_TERM, fma / FP32_PER_TERM) * n_sm * clk * 1e6
    bound = "mufu" if mufu / MUFU_PER_TERM <= fma / FP32_PER_TERM else "fp32"
    form_name, mufu_pt, fp32_pt = FORMS[mode]
    form_peak = min(mufu / mufu_pt, fma / fp32_pt) * n_sm * clk * 1e6
    form_bound = "mufu" if mufu / mufu_pt <= fma / fp32_pt else "fp32"
    traffic = profiled_traffic(args.config, n_pix, launch)
    achieved = terms / (split_ms * 1e-3)
    gpu_launches = args.steps * (8 + int(bool(ftab)))

    configs = configs_leg(args, dev) if (rank == 0 and not args.no_configs) else None
    scan = scan_leg(args, dev) if (rank == 0 and args.scan_frames > 0) else None
    surr = surrogate_leg(args, dev) if (rank == 0 and not args.no_surrogate) else None
    if rank == 0:
        cpu = cpu_baseline(w) if not args.no_cpu else None
        line = {
            "metric": METRIC,
            "value": value, "unit": "Gatom*pixel/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 origins and reduction)",
            "data": "synthetic",
            "config": {"workload": args.config, "atoms": n_atoms, "pixels": n_pix,
                       "terms_per_step": terms, "tile_atoms": B._kernel_tile_atoms,
                       "launch": launch, "fresnel_term": bool(fresnel), "factor_table": bool(ftab),
                       "l2": "inputs larger than L2 (positions + tiles ~300 MB); no flush",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": terms * world / e2e_s / 1e9, "unit": "Gatom*pixel/s",
                    "seconds": e2e_s, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "pixels_kept_from_the_previous_call": bool(getattr(B, "last_pixels_cached",
                                                                       False))},
            "gpu_launches": gpu_launches,
            "roofline": {"bound": form_bound, "achieved": achieved / 1e9, "peak": form_peak / 1e9,
                         "unit": "Gterm/s", "frac": achieved / form_peak,
                         "traffic": traffic["bytes_per_launch"] if traffic else None,
                         "traffic_source": traffic,
                         "peak_source": f"executed form ({form_name}): min(MUFU sin/cos "
                                        f"{mufu:.2f}/clk/SM / {mufu_pt} per term, FP32 "
                                        f"{fma:.1f}/clk/SM / {fp32_pt} per term); both pipe rates "
                                        f"measured on this GPU by mk_probe_throughput (the measured "
                                        f"peaks file carries no FP32 or MUFU figure), x {n_sm} SMs "
                                        f"x {clk:.0f} MHz ({peak_src} max clock)",
                         "fp32_lane_tops": achieved * fp32_pt / 1e12,
                         "fp32_lane_peak_tops": fma * n_sm * clk * 1e6 / 1e12,
                         "canonical": {"mufu_per_term": MUFU_PER_TERM, "fp32_per_term": FP32_PER_TERM,
                                       "bound": bound, "peak": peak_terms / 1e9,
                                       "ratio": achieved / peak_terms,
                                       "note": "achieved over the canonical split-phase term's "
                                               "bound (2 MUFU + 12 FP32 per term): an algorithmic "
                                               "savings ratio, not a roofline fraction -- the "
                                               "executed form shares sin/cos between pixels"},
                         "pipe_probe_ops_per_clk_per_sm": pipes,
                         "split_kernel_ms": split_ms},
            "fp64_plain": {"value": fp64_rate, "unit": "Gatom*pixel/s",
                           "subset": f"{m} pixels spread over the whole detector, all atoms",
                           "speedup_fp32_vs_fp64": (achieved / 1e9) / fp64_rate},
            "accuracy": {"rel_err_max_over_peak": chk["rel_err_max_over_peak"],
                         "rel_err_l2": chk["rel_err_l2"],
                         "rel_err_corners_and_edge_midpoints":
                             chk["rel_err_corners_and_edge_midpoints"],
                         "rel_err_local_max_where_I_ge_1e-3_peak":
                             chk["rel_err_local_max_where_I_ge_1e-3_peak"],
                         "pixels": m,
                         "reference": f"FP64 plain GPU kernel at {m} pixels spread over the whole "
                                      f"detector: the 4 corners, the 4 edge midpoints, the centre "
                                      f"and a {args.fp64_grid} x {args.fp64_grid} edge-to-edge grid",
                         "budget": 1e-4},
            "split_budget": {k: float(v) for k, v in diag.items()},
            "autotune": [[float(t), c] for t, c in tune_tbl] if tune_tbl else [],
            "clocks": clocks,
            "cpu_baseline": cpu,
            "configs": configs,
            "scan": scan,
            "surrogate_scan": surr,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="nacl_screw_8m")
    ap.add_argument("--tile-atoms", type=int, default=0,
                    help="atoms per tile (power of two, 128-4096; 0: the beam's default 512)")
    ap.add_argument("--fp64-grid", type=int, default=32,
                    help="side of the edge-to-edge pixel grid the FP64 reference is computed on")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip configs 1 and 3 (end to end through the entry point)")
    ap.add_argument("--no-surrogate", action="store_true",
                    help="skip the surrogate-assisted scan leg (101 x 101 frames)")
    ap.add_argument("--surrogate-verify", type=int, default=64,
                    help="unjudged predicted frames checked against the exact sum (untimed)")
    ap.add_argument("--surrogate-exact-all", action=argparse.BooleanOptionalAction, default=True,
                    help="also compute every frame exactly: the measured exact-only scan time "
                         "and the error of every returned frame (the exact scan takes ~2 min; "
                         "--no-surrogate-exact-all estimates it from the exact launch instead "
                         "and checks --surrogate-verify sampled frames)")
    ap.add_argument("--no-pairs", action="store_true",
                    help="one sin/cos per term (the pixel-pair and quad forms off)")
    ap.add_argument("--launch", default="",
                    help="fixed launch shape 'pixels_per_thread,threads,mode' (mode 0 one sin/cos "
                         "per term, 1 pairs, 2 quads, 3 octets, 4 squares; clamped to what the geometry "
                         "allows) "
                         "instead of the autotuner's")
    ap.add_argument("--no-quads", action="store_true",
                    help="at most one sin/cos per pixel pair (the 2x2 quad and octet forms off)")
    ap.add_argument("--no-octets", action="store_true",
                    help="at most the 2x2 quad form (the 2x4 octet and 4x4 square forms off)")
    ap.add_argument("--no-factor-table", action="store_true",
                    help="the scattering factor per (tile, pixel) instead of the per-(species, "
                         "pixel) table")
    ap.add_argument("--no-squares", action="store_true",
                    help="at most the 2x4 octet form (the 4x4 square form off)")
    ap.add_argument("--scan-frames", type=int, default=724,
                    help="frames of the batched-scan leg (0: skip; the configuration has 724)")
    ap.add_argument("--profile-gemm", action="store_true",
                    help="kernel-profile case of the surrogate's tcgen05 GEMM shapes (no bench line)")
    ap.add_argument("--profile", action="store_true",
                    help="kernel-profile run: cached launch shape, timed steps only")
    args = ap.parse_args()
    if args.profile_gemm:
        gemm_profile_case()
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
