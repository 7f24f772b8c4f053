"""``scan_nD``: the reference's N-dimensional motor scan, run as one batched launch.

Same arguments and result dict as experiment.scan_nD (Experiment.py:35-406):
1..3 axes over stage motors and/or detector axes (two_theta / 2theta / tth,
eta, distance), absolute or relative ranges, couplings (source motor ->
[(target, ratio)], ratio a number or "a:b" meaning b/a), and per step the
summed intensity. The reference moves the motors and runs one full
exposure per step; here the same motor walk only RECORDS each step's
stage transform and detector pixels, and every step is then computed in a
single persistent launch (``mosaic_gb300.scan.BatchedScan``). Plotting is
not part of this library: the figure arguments are accepted and ignored.

Motor and detector states are restored after the walk.
"""
from __future__ import annotations

import copy

import numpy as np

from . import engine
from .geometry import StaticStage
from .scan import BatchedScan, Frame, roi_indices

DET_AXES = {"two_theta": "two_theta", "2theta": "two_theta", "tth": "two_theta", "eta": "eta",
            "distance": "distance"}


def _canon(name):
    return DET_AXES.get(str(name).strip().lower())


def parse_ratio(r):
    if isinstance(r, (int, float)):
        return float(r)
    s = str(r)
    if ":" in s:
        a, b = (float(x.strip()) for x in s.split(":"))
        if a == 0.0:
            raise ValueError("Invalid coupling ratio a:b with a=0.")
        return b / a
    return float(s)


def axis_values(start, stop, step, current=0.0, relative=False):
    """Axis samples as the reference builds them (Experiment.py:238-253)."""
    a0, a1 = (current + start, current + stop) if relative else (float(start), float(stop))
    step = float(step)
    if step == 0.0:
        raise ValueError("Step size is 0.")
    if (a1 - a0) * step < 0.0:
        raise ValueError("Step sign does not move from start to stop.")
    count = int(np.floor(abs((a1 - a0) / step) + 1e-12)) + 1
    vals = a0 + step * np.arange(count, dtype=float)
    if count == 0 or (step > 0 and vals[-1] < a1 - 1e-10) or (step < 0 and vals[-1] > a1 + 1e-10):
        vals = np.append(vals, a1)
    return vals


def scan_frames(detector, stage, ranges, stepsizes, motors, degrees=True, scan_mode="absolute",
                couplings=None, rois=None):
    """Walk the scan grid like the reference and record one Frame per step.

    Returns (axis_vals, grid_shape, frames). ``rois``: None (full detector),
    an int side for every step, or a callable step_index -> side.
    """
    n = len(motors)
    if n < 1 or n > 3:
        raise ValueError(f"scan_nD supports 1, 2, or 3 axes. Got {n}.")
    if not (len(stepsizes) == len(ranges) == len(motors)):
        raise ValueError("ranges, stepsizes, and motors must have same length.")
    det = copy.deepcopy(detector)
    st = copy.deepcopy(stage)

    def current(m):
        c = _canon(m)
        if c == "two_theta":
            return np.degrees(det.two_theta) if degrees else float(det.two_theta)
        if c == "eta":
            return np.degrees(det.eta) if degrees else float(det.eta)
        if c == "distance":
            return float(det.distance)
        i = st.motor_index(str(m))
        v = float(st.motor_value[i])
        return np.degrees(v) if (st.motor_types[i] == "R" and degrees) else v

    def move(m, delta):
        c = _canon(m)
        if c == "two_theta":
            det.position_detector_relative(0.0, delta, 0.0, degrees=degrees)
        elif c == "eta":
            det.position_detector_relative(0.0, 0.0, delta, degrees=degrees)
        elif c == "distance":
            det.position_detector_relative(delta, 0.0, 0.0, degrees=degrees)
        else:
            st.set_single_motor_value_relative(str(m), delta, degrees=degrees)

    for m in motors:
        if _canon(m) is None:
            st.motor_index(str(m))                       # raises for unknown names
    key = lambda m: _canon(m) or str(m)
    primary = {key(m) for m in motors}
    coup = {}
    for src, lst in (couplings or {}).items():
        coup[key(src)] = [(key(t), parse_ratio(r)) for t, r in lst]
    rel = str(scan_mode).lower() == "relative"
    axes = [axis_values(r[0], r[1], s, current(m), rel) for r, s, m in zip(ranges, stepsizes, motors)]
    shape = tuple(len(a) for a in axes)
    frames = []
    for k, idx in enumerate(np.ndindex(*shape)):
        for j, m in enumerate(motors):
            target = float(axes[j][idx[j]])
            delta = target - current(m)
            if abs(delta) > 1e-12 * max(1.0, abs(target)):
                move(m, delta)
                for tgt, ratio in coup.get(key(m), []):
                    if tgt not in primary:
                        move(tgt, ratio * delta)
        coords = np.asarray(det.pixel_coordinates)
        side = rois(k) if callable(rois) else rois
        if side is not None:
            sel, fshape = roi_indices(det.shape, side)
            coords = coords[:, sel]
        else:
            fshape = tuple(det.shape)
        frames.append(Frame(st.rotation.copy(), st.translation.copy(), coords.copy(), fshape))
    return axes, shape, frames


def scan_nD(sample, beam, detector, stage, ranges, stepsizes, motors, degrees=True,
            scan_mode="absolute", optics=None, couplings=None, per_step_outputs=("Intensity",),
            plot_in_angle_space=False, show_plots=False, save_dir=None, adi_kwargs=None,
            prop_kwargs=None, step_callback=None, rois=None, return_scan=False):
    """N-D scan (Experiment.py:35-406) computed in one batched launch.

    Returns dict(axes, motor_names, sum_intensity, step_count, summary_image)
    like the reference; with ``return_scan`` also the BatchedScan (per-frame
    fields on the device)."""
    if optics is not None:
        raise NotImplementedError("optics stacks per scan step are not provided")
    kw = dict(apply_polarization=False, spherical_decay=False, remove_forward=False)
    sc = dict((adi_kwargs or {}).get("sc_kwargs", {}))
    kw.update({k: v for k, v in sc.items() if k in kw})
    axes, shape, frames = scan_frames(detector, stage, ranges, stepsizes, motors, degrees,
                                      scan_mode, couplings, rois)
    per_frame = bool(sc.get("use_depth_ein")) or engine.analyser_kind(sc.get("analyser_mode"))
    scan = None
    if per_frame:
        # The analyser and the depth-dependent field change with every pose:
        # one exposure per step through the single-exposure kernels, as the
        # reference's own scan loop does (Experiment.py:285-336).
        one = {k: sc[k] for k in ("analyser_mode", "analyser_acceptance_angle_rad",
                                  "analyser_darwin_halfwidth_rad", "use_depth_ein") if k in sc}
        sums = np.empty(len(frames))
        for i, f in enumerate(frames):
            st = StaticStage(f.rotation, f.translation)
            A = beam.interact_beam_gpu(sample, np.asarray(f.pixels), f.shape, st,
                                       return_double=True, **kw, **one)
            sums[i] = float((np.abs(A) ** 2).sum())
        sums = sums.reshape(shape)
    else:
        scan = BatchedScan(beam, sample, frames, **kw)
        scan.run()
        sums = scan.sum_intensity().reshape(shape)
    if step_callback is not None:
        for k, idx in enumerate(np.ndindex(*shape)):
            step_callback({"step": k + 1, "total": len(frames), "index": tuple(int(i) for i in idx),
                           "position": ", ".join(f"{m}={axes[j][idx[j]]:.6g}" for j, m in enumerate(motors)),
                           "sum_intensity": float(sums[idx]), "figures": {}, "image_paths": {}})
    res = {"axes": axes, "motor_names": list(motors), "sum_intensity": sums,
           "step_count": len(frames), "summary_image": None}
    if return_scan:
        res["scan"] = scan
    return res
