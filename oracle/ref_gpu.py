"""The reference's GPU general kernel on this GPU -- TEST INFRASTRUCTURE ONLY.

Nothing in ``mosaic_gb300`` imports this module. It loads the libraries
``oracle/ref_build.py`` compiles from the reference's own kernel source
(``interaction_kernal``, Beam.py:1698-2415) and stages inputs the way the
reference's ``interact_beam_gpu`` does for that kernel (``_stage_general_subchunk``,
Beam.py:1541-1599; launch Beam.py:6327-6366): float32 positions in metres
with one global origin, per-atom k, Waasmaier-Kirfel rows, f0(0), f'+if''
and incident amplitude, float32 pixel coordinates in metres. It is the
comparator "the reference's kernel on the GB300" and pins the analyser
(which the reference applies only in this kernel) to the reference.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import ref_build

_libs = {}


def series_mode(a_max_m, r0_min_m, k, phi_tol=1e-3, safety_t=0.5):
    """The reference's choice of series or exact form and of the series
    order (``_estimate_required_series_terms`` and ``_select_series_mode_once``,
    Beam.py:1063-1130, 1158-1202): the smallest N whose first omitted term
    k R0 |C_{N+1}| t^(N+1) is within the phase tolerance, t = 2 rho + rho^2,
    rho = a_max / R0_min; the exact form when t >= 0.5 or no N <= 31 fits.
    Returns (use_series, N)."""
    if not (r0_min_m > 0.0):
        return False, 1
    rho = float(a_max_m) / float(r0_min_m)
    t = 2.0 * rho + rho * rho
    if not (t < 1.0) or not (t < safety_t):
        return False, 1
    C, tk, terms = 0.5, t, [(0.5 * t, 1)]
    for kk in range(2, 33):
        C = C * ((0.5 - (kk - 1.0)) / kk)
        tk = tk * t
        terms.append((abs(C) * tk, kk))
    for N in range(1, 32):
        if float(k) * float(r0_min_m) * terms[N][0] <= float(phi_tol):
            return True, N
    return False, 1


def library_mode(use_series, N):
    """The built library for a series setting: the smallest built series
    order >= N (more terms only add accuracy), or the exact form."""
    if not use_series:
        return "exact"
    built = sorted(int(m[1:]) for m in ref_build.GPU_MODES if m != "exact")
    for b in built:
        if b >= N:
            return f"s{b}"
    return "exact"


def lib(mode):
    """ctypes handle of libref_general_<mode>.so, or None when not built."""
    if mode in _libs:
        return _libs[mode]
    built = ref_build.build_gpu()
    so = built.get(mode)
    if so is None or not os.path.exists(so):
        _libs[mode] = None
        return None
    L = ctypes.CDLL(so)
    vp, fl, it = ctypes.c_void_p, ctypes.c_float, ctypes.c_int
    L.mkref_general.restype = it
    L.mkref_general.argtypes = [it] + [vp] * 13 + [vp, it, it, it, it, it, fl, it, fl, fl, fl,
                                                   fl, fl, vp, vp]
    _libs[mode] = L
    return L


def available():
    return lib("exact") is not None


def pol_rate(pol):
    """The pol_perp_rate rho that gives polarization (p, e) in the kernel
    (p = |2 rho - 1|, e = y for rho >= 0.5 else z; Beam.py:1948-1957), or None
    when e is neither axis."""
    p, ex, ey, ez = (float(v) for v in pol)
    if p == 0.0:
        return 0.5
    if abs(ey - 1.0) < 1e-12 and abs(ex) < 1e-12 and abs(ez) < 1e-12:
        return 0.5 + 0.5 * p
    if abs(ez - 1.0) < 1e-12 and abs(ex) < 1e-12 and abs(ey) < 1e-12:
        return 0.5 - 0.5 * p
    return None


def general(pos_m, wk, f0z, anom, amp, cxyz_m, ny, nz, k, remove_forward=False,
            apply_pol=False, pol_rate_value=1.0, decay=False, analyser=None, mode=None,
            device="cuda", sub_atoms=65536, stream=None, a_max_m=None, phi_tol=1e-3):
    """Run the reference's kernel: per-atom float32 inputs (positions (N,3)
    metres relative to the one global origin, WK rows (N,11), f0(0) (N,),
    complex f'+if'' (N,) and incident amplitude (N,)), pixel coordinates
    (3, P) metres. ``analyser`` = (kind 1 top-hat / 2 Darwin, centre (3,)
    metres, acceptance [rad], half-width [rad]). ``mode`` "sN" / "exact"
    (None: the reference's own choice for this geometry, ``series_mode``).
    Returns the complex64 (P,) field as the kernel accumulates it, and the
    mode used."""
    import torch
    n = int(np.asarray(pos_m).shape[0])
    P = int(ny) * int(nz)
    dev = torch.device(device)
    f32 = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32)).to(dev)
    pos = np.asarray(pos_m, dtype=np.float32).reshape(n, 3)
    c = np.asarray(cxyz_m, dtype=np.float32).reshape(3, P)
    if mode is None:
        a_max = float(np.linalg.norm(pos.astype(np.float64), axis=1).max()) if a_max_m is None \
            else float(a_max_m)
        r0 = float(np.linalg.norm(c.astype(np.float64), axis=0).min())
        mode = library_mode(*series_mode(a_max, r0, k, phi_tol))
    L = lib(mode)
    if L is None:
        raise RuntimeError(f"the reference GPU kernel ({mode}) is not built")
    px, py, pz = (f32(pos[:, i]) for i in range(3))
    kx = torch.full((n,), float(np.float32(k)), dtype=torch.float32, device=dev)
    kyz = torch.zeros(n, dtype=torch.float32, device=dev)
    c64 = lambda a: torch.view_as_real(torch.as_tensor(
        np.ascontiguousarray(np.asarray(a).astype(np.complex64)).reshape(n))).to(dev).contiguous()
    amp_t, anom_t = c64(amp), c64(anom)
    wk_t = f32(np.asarray(wk).reshape(n, 11))
    f0z_t = f32(np.asarray(f0z).reshape(n))
    x, y, z = (f32(c[i]) for i in range(3))
    field = torch.zeros((P, 2), dtype=torch.float32, device=dev)
    zeros3 = torch.zeros(3, dtype=torch.float32, device=dev)
    kind, cen, acc, hw = 0, (0.0, 0.0, 0.0), 0.0, 0.0
    if analyser is not None:
        kind, cen, acc, hw = int(analyser[0]), analyser[1], float(analyser[2]), float(analyser[3])
    s = stream or torch.cuda.current_stream(dev)
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())
    for a0 in range(0, n, int(sub_atoms)):
        a1 = min(n, a0 + int(sub_atoms))
        off4, off8, off44 = a0 * 4, a0 * 8, a0 * 44
        rc = L.mkref_general(
            a1 - a0, ctypes.c_void_p(kx.data_ptr() + off4), ctypes.c_void_p(kyz.data_ptr() + off4),
            ctypes.c_void_p(kyz.data_ptr() + off4), ctypes.c_void_p(px.data_ptr() + off4),
            ctypes.c_void_p(py.data_ptr() + off4), ctypes.c_void_p(pz.data_ptr() + off4),
            ctypes.c_void_p(amp_t.data_ptr() + off8), ctypes.c_void_p(anom_t.data_ptr() + off8),
            ctypes.c_void_p(wk_t.data_ptr() + off44), ctypes.c_void_p(f0z_t.data_ptr() + off4),
            ptr(x), ptr(y), ptr(z), ptr(field), int(ny), int(nz), int(bool(remove_forward)),
            int(bool(apply_pol)), int(bool(decay)), float(pol_rate_value), kind,
            float(cen[0]), float(cen[1]), float(cen[2]), acc, hw, ptr(zeros3),
            ctypes.c_void_p(s.cuda_stream))
        if rc != 0:
            raise RuntimeError(f"reference kernel launch failed: cudaError {rc}")
    s.synchronize()
    f = field.cpu().numpy()
    return (f[:, 0] + 1j * f[:, 1]).astype(np.complex64), mode
