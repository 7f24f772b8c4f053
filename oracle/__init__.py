"""CPU oracle for the kinematic scattering path -- TEST INFRASTRUCTURE ONLY.

Nothing in the product (``mosaic_gb300``) imports this package. Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
it, and only as the checker (or as the timed CPU baseline).

Contents
--------
* ``kin_oracle.c`` -- FP64 C restatement of the reference CPU kernel
  ``compute_scattering_cffi`` (MOSAIC ``Beam.py:663-816``), threaded over atom
  slices summed in slice order (``Beam.py:5941-5955``), plus the free-space
  propagator multiply (``Beam.py:4747-4834``).
* ``scatter_ref`` -- the reference's OWN CPU kernel, ``compute_scattering_cffi``,
  compiled from its source by ``oracle/ref_build.py`` into ``oracle/_ref/``
  when a reference checkout (or its extracted source) is present: the
  timed CPU baseline of the reference, threaded over atom slices summed in
  slice order as ``interact_beam_cpu`` does (``Beam.py:5933-5955``).
* ``ref_tables`` / ``ein_bilinear`` / ``polarization_state`` /
  ``interact_cpu`` below -- NumPy restatements of the reference host logic
  around that kernel (``Beam.py:31-47``, ``117-149``, ``503-615``, ``956-1045``,
  ``5621-5956``).

Pinning: every function here is checked against fixtures produced by running
the reference itself (``tests/golden/make_golden.py``), see
``tests/test_oracle_golden.py``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "kin_oracle.c")
_SO = os.path.join(_HERE, "_ref", "libkin_oracle.so")
_lib = None

R_E = 2.81794092e-15          # classical electron radius [m] (Beam.py:704)
H_PLANCK = 6.62607015e-34     # SI constants of beam.__init__ (Beam.py:98-101)
C_LIGHT = 299792458
Q_E = 1.602176634e-19


def build(force: bool = False) -> str:
    """Compile kin_oracle.c into oracle/_ref/libkin_oracle.so, and the
    reference's own CPU kernel where its source is available
    (oracle/ref_build.py).

    gcc -O3 with -ffp-contract=off: without contraction the x86 and Arm builds
    round every operation identically. The absolute phase k (x + r) is ~1e10 rad,
    where one double ulp is ~2e-6 rad, so an FMA-contracted build (as the
    reference's -march=native cffi build is) differs from an uncontracted one
    by ~1e-6 relative in the summed field.
    """
    os.makedirs(os.path.dirname(_SO), exist_ok=True)
    if (not force and os.path.exists(_SO)
            and os.path.getmtime(_SO) >= os.path.getmtime(_SRC)):
        _build_ref()
        return _SO
    tmp = _SO + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O3", "-ffp-contract=off", "-std=c11", "-shared", "-fPIC", "-pthread",
                           _SRC, "-o", tmp, "-lm"])
    os.replace(tmp, _SO)
    _build_ref()
    return _SO


def _build_ref():
    """The reference's own kernels where their source is available: the CPU
    kernel (gcc) and the GPU general kernel (nvcc, for the comparator)."""
    from . import ref_build
    for step in (ref_build.build, ref_build.build_gpu):
        try:
            step()
        except (OSError, subprocess.CalledProcessError, ValueError, RuntimeError):
            pass


_ref_lib = None


def ref_lib():
    """The reference's own compute_scattering_cffi (ctypes), or None when it
    could not be built here (no reference checkout and no extracted source)."""
    global _ref_lib
    if _ref_lib is None:
        from . import ref_build
        try:
            so = ref_build.build()
        except (OSError, subprocess.CalledProcessError, ValueError, RuntimeError):
            so = None
        if so is None:
            return None
        L = ctypes.CDLL(so)
        dp = ctypes.POINTER(ctypes.c_double)
        fp = ctypes.POINTER(ctypes.c_float)
        L.compute_scattering_cffi.restype = ctypes.c_int
        L.compute_scattering_cffi.argtypes = [
            ctypes.c_int, dp, fp, fp, ctypes.c_int, fp, fp, fp, fp, ctypes.c_int, ctypes.c_int,
            dp, dp, dp, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double,
            ctypes.c_double, ctypes.c_double, ctypes.c_int, fp, fp]
        _ref_lib = L
    return _ref_lib


def scatter_ref(pos_m, wk, f0z, anom_re, anom_im, amp_re, amp_im, cx, cy, cz, k, ny, nz,
                remove_forward=False, apply_pol=False, pol=(0.0, 0.0, 1.0, 0.0), decay=False,
                n_threads=None, slice_atoms=None):
    """The reference's own CPU kernel on atom slices, ``n_threads`` at a time
    (ctypes releases the GIL), each slice into its own float32 buffers and
    the slices summed in order (Beam.py:5933-5955). Same arguments as
    ``scatter_f64`` (no Debye-Waller factor or analyser: the reference's CPU
    kernel has neither). Returns complex128 (ny*nz,)."""
    from concurrent.futures import ThreadPoolExecutor
    L = ref_lib()
    if L is None:
        raise RuntimeError("the reference CPU kernel is not built (oracle/ref_build.py)")
    n = int(np.asarray(pos_m).shape[0])
    P = int(ny) * int(nz)
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    pos = f64(pos_m).reshape(n, 3)
    wk = f32(wk).reshape(n, 11)
    f0z, ar, ai, er, ei = (f32(v).reshape(n) for v in (f0z, anom_re, anom_im, amp_re, amp_im))
    cx, cy, cz = (f64(v).reshape(P) for v in (cx, cy, cz))
    nt = int(n_threads or os.cpu_count() or 1)
    sl = int(slice_atoms or max(1000, -(-max(n, 1) // nt)))

    def run(a0, a1):
        o_r = np.zeros(P, np.float32)
        o_i = np.zeros(P, np.float32)
        rc = L.compute_scattering_cffi(
            a1 - a0, _p(pos[a0:a1], ctypes.c_double), _p(wk[a0:a1], ctypes.c_float),
            _p(f0z[a0:a1], ctypes.c_float), int(bool(remove_forward)),
            _p(ar[a0:a1], ctypes.c_float), _p(ai[a0:a1], ctypes.c_float),
            _p(er[a0:a1], ctypes.c_float), _p(ei[a0:a1], ctypes.c_float), int(ny), int(nz),
            _p(cx, ctypes.c_double), _p(cy, ctypes.c_double), _p(cz, ctypes.c_double), float(k),
            int(bool(apply_pol)), float(pol[0]), float(pol[1]), float(pol[2]), float(pol[3]),
            int(bool(decay)), _p(o_r, ctypes.c_float), _p(o_i, ctypes.c_float))
        if rc != 0:
            raise MemoryError("reference CPU kernel could not allocate its work buffers")
        return o_r.astype(np.float64) + 1j * o_i.astype(np.float64)

    out = np.zeros(P, np.complex128)
    bounds = [(a, min(a + sl, n)) for a in range(0, n, sl)]
    with ThreadPoolExecutor(max_workers=max(1, min(nt, len(bounds)))) as ex:
        for f in [ex.submit(run, a, b) for a, b in bounds]:
            out += f.result()
    return out


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_SO)
        dp = ctypes.POINTER(ctypes.c_double)
        fp = ctypes.POINTER(ctypes.c_float)
        L.mko_scatter_f64.restype = ctypes.c_int
        L.mko_scatter_f64.argtypes = [
            ctypes.c_int64, dp, fp, fp, ctypes.c_int, fp, fp, fp, fp, fp,
            ctypes.c_int, ctypes.c_int, dp, dp, dp, ctypes.c_double, ctypes.c_int,
            ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
            ctypes.c_int, ctypes.c_int, dp, ctypes.c_double, ctypes.c_double, dp, dp, ctypes.c_int]
        L.mko_prop_mul_f64.restype = None
        L.mko_prop_mul_f64.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, dp]
        _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def scatter_f64(pos_m, wk, f0z, anom_re, anom_im, amp_re, amp_im, cx, cy, cz, k,
                ny, nz, remove_forward=False, apply_pol=False,
                pol=(0.0, 0.0, 1.0, 0.0), decay=False, dw_b=None, n_threads=None,
                analyser=None):
    """FP64 kinematic sum (compute_scattering_cffi semantics, double output).

    Args mirror ``Beam.py:631-651``: positions (N,3) metres, per-atom WK rows
    (N,11), f0(0), f'/f'' and incident amplitude; pixel coordinates in metres.
    ``pol`` = (p, ex, ey, ez). ``analyser`` = (kind 1 top-hat / 2 Darwin,
    axis (3,), acceptance [rad], half-width [rad]), the general GPU kernel's
    factor (Beam.py:2350-2378). Returns complex128 (ny*nz,).
    """
    L = lib()
    n = int(np.asarray(pos_m).shape[0])
    P = int(ny) * int(nz)
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    pos = f64(pos_m).reshape(n, 3)
    wk = f32(wk).reshape(n, 11)
    f0z, ar, ai, er, ei = (f32(v).reshape(n) for v in (f0z, anom_re, anom_im, amp_re, amp_im))
    dwb = None if dw_b is None else f32(dw_b).reshape(n)
    cx, cy, cz = (f64(v).reshape(P) for v in (cx, cy, cz))
    out_r = np.zeros(P)
    out_i = np.zeros(P)
    nt = int(n_threads or os.cpu_count() or 1)
    an_kind, an_axis, an_acc, an_hw = 0, np.zeros(3), 0.0, 0.0
    if analyser is not None and int(analyser[0]):
        an_kind = int(analyser[0])
        an_axis = f64(analyser[1]).reshape(3)
        an_acc, an_hw = float(analyser[2]), float(analyser[3])
    an_axis = f64(an_axis)
    rc = L.mko_scatter_f64(
        n, _p(pos, ctypes.c_double), _p(wk, ctypes.c_float), _p(f0z, ctypes.c_float),
        int(bool(remove_forward)), _p(ar, ctypes.c_float), _p(ai, ctypes.c_float),
        _p(er, ctypes.c_float), _p(ei, ctypes.c_float),
        None if dwb is None else _p(dwb, ctypes.c_float),
        int(ny), int(nz), _p(cx, ctypes.c_double), _p(cy, ctypes.c_double),
        _p(cz, ctypes.c_double), float(k), int(bool(apply_pol)),
        float(pol[0]), float(pol[1]), float(pol[2]), float(pol[3]), int(bool(decay)),
        an_kind, _p(an_axis, ctypes.c_double), an_acc, an_hw,
        _p(out_r, ctypes.c_double), _p(out_i, ctypes.c_double), nt)
    if rc != 0:
        raise MemoryError("oracle scatter could not allocate its work buffers")
    return out_r + 1j * out_i


def prop_mul_f64(F, ky, kz, k, z, kga=None, kgy=0.0, kgz=0.0):
    """Free-space transfer-function multiply (Beam.py:4747-4834), FP64, returns a copy."""
    L = lib()
    G = np.ascontiguousarray(F, dtype=np.complex128).copy()
    nz, ny = G.shape
    ky = np.ascontiguousarray(ky, dtype=np.float64)
    kz = np.ascontiguousarray(kz, dtype=np.float64)
    L.mko_prop_mul_f64(int(ny), int(nz), _p(ky, ctypes.c_double), _p(kz, ctypes.c_double),
                       float(k), float(z), float(k if kga is None else kga), float(kgy),
                       float(kgz), G.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return G


# --------------------------------------------------------------------------
# NumPy restatements of the host logic around the kernel
# --------------------------------------------------------------------------
def polarization_state(pol_perp_rate=0.5, pol_direction=None, pol_degree=None,
                       direction=(1.0, 0.0, 0.0)):
    """(p, ex, ey, ez) as ``beam._polarization_state`` (Beam.py:117-149, 31-47)."""
    khat = np.asarray(direction, dtype=np.float64)
    khat = khat / np.linalg.norm(khat)
    rho = float(np.clip(pol_perp_rate, 0.0, 1.0))
    p_rate = abs(2.0 * rho - 1.0)
    e_rate = np.array([0.0, 1.0, 0.0]) if rho >= 0.5 else np.array([0.0, 0.0, 1.0])
    p = p_rate if pol_degree is None else float(np.clip(pol_degree, 0.0, 1.0))
    e = e_rate if pol_direction is None else np.asarray(pol_direction, dtype=np.float64).reshape(3)
    e = e - np.dot(e, khat) * khat
    if np.linalg.norm(e) < 1e-12:
        for axis in (np.array([0.0, 1.0, 0.0]), np.array([0.0, 0.0, 1.0])):
            e = axis - np.dot(axis, khat) * khat
            if np.linalg.norm(e) >= 1e-12:
                break
    e = e / np.linalg.norm(e)
    return float(p), float(e[0]), float(e[1]), float(e[2])


def anomalous(energy, table):
    """f' + i f'' by linear interpolation in energy, end segment extended
    (Beam.py:569-597). ``table`` is (N,3) [E, f1, f2] float32."""
    E = table[:, 0]
    idx = int(np.searchsorted(E, energy))
    idx = min(max(idx, 1), len(E) - 1)
    E0, E1 = E[idx - 1], E[idx]
    w = (energy - E0) / ((E1 - E0) if E1 > E0 else 1e-20)
    f1 = table[idx - 1, 1] + (table[idx, 1] - table[idx - 1, 1]) * w
    f2 = table[idx - 1, 2] + (table[idx, 2] - table[idx - 1, 2]) * w
    return complex(f1, f2)


def ein_bilinear(pos, E0, du, dv, uc, vc, e1=(0, 1, 0), e2=(0, 0, 1)):
    """Per-atom incident amplitude by bilinear sampling of E0 with tau = phi = 0,
    zero outside the grid (Beam.py:956-1045). pos (N,3) float32 Angstrom."""
    pos = np.asarray(pos, dtype=np.float32)
    e1 = np.asarray(e1, dtype=np.float32)
    e2 = np.asarray(e2, dtype=np.float32)
    N = pos.shape[0]
    out = np.zeros(N, dtype=np.complex64)
    NyB, NzB = E0.shape
    au = pos[:, 0] * e1[0] + pos[:, 1] * e1[1] + pos[:, 2] * e1[2]
    av = pos[:, 0] * e2[0] + pos[:, 1] * e2[1] + pos[:, 2] * e2[2]
    iu = au / float(du) + float(uc)
    iv = av / float(dv) + float(vc)
    inb = (iu >= 0.0) & (iu <= NyB - 1) & (iv >= 0.0) & (iv <= NzB - 1)
    if not np.any(inb):
        return out
    iu, iv = iu[inb], iv[inb]
    i0 = np.floor(iu).astype(np.int64)
    j0 = np.floor(iv).astype(np.int64)
    i1 = np.clip(i0 + 1, 0, NyB - 1)
    j1 = np.clip(j0 + 1, 0, NzB - 1)
    fu = (iu - i0).astype(np.float32)
    fv = (iv - j0).astype(np.float32)
    Ef = np.asarray(E0, dtype=np.complex64).ravel()
    val = (Ef[i0 * NzB + j0] * ((1 - fu) * (1 - fv)) + Ef[i0 * NzB + j1] * ((1 - fu) * fv)
           + Ef[i1 * NzB + j0] * (fu * (1 - fv)) + Ef[i1 * NzB + j1] * (fu * fv))
    out[inb] = val.astype(np.complex64)
    return out


def ein_depth(pos, E0, tau, phi, du, dv, uc, vc, s_min, s_max, e1=(0, 1, 0), e2=(0, 0, 1),
              khat=(1, 0, 0)):
    """Per-atom incident amplitude with the depth-dependent transmission
    (Beam.py:956-1045): E0, tau and phi sampled bilinearly at the atom's
    beam-grid position, Ein = E0 exp(-f tau) exp(i f phi) with
    f = clip((khat.pos - s_min) / (s_max - s_min), 0, 1); zero outside the
    grid. float32 arithmetic in the reference's order."""
    pos = np.asarray(pos, dtype=np.float32)
    e1, e2, khat = (np.asarray(v, dtype=np.float32) for v in (e1, e2, khat))
    N = pos.shape[0]
    out = np.zeros(N, dtype=np.complex64)
    NyB, NzB = E0.shape
    au = pos[:, 0] * e1[0] + pos[:, 1] * e1[1] + pos[:, 2] * e1[2]
    av = pos[:, 0] * e2[0] + pos[:, 1] * e2[1] + pos[:, 2] * e2[2]
    iu = au / float(du) + float(uc)
    iv = av / float(dv) + float(vc)
    inb = (iu >= 0.0) & (iu <= NyB - 1) & (iv >= 0.0) & (iv <= NzB - 1)
    if not np.any(inb):
        return out
    iu, iv = iu[inb], iv[inb]
    i0 = np.floor(iu).astype(np.int64)
    j0 = np.floor(iv).astype(np.int64)
    i1 = np.clip(i0 + 1, 0, NyB - 1)
    j1 = np.clip(j0 + 1, 0, NzB - 1)
    fu = (iu - i0).astype(np.float32)
    fv = (iv - j0).astype(np.float32)
    w00, w01, w10, w11 = (1 - fu) * (1 - fv), (1 - fu) * fv, fu * (1 - fv), fu * fv
    r00, r01, r10, r11 = i0 * NzB + j0, i0 * NzB + j1, i1 * NzB + j0, i1 * NzB + j1
    tf = np.asarray(tau, np.float32).ravel()
    pf = np.asarray(phi, np.float32).ravel()
    Ef = np.asarray(E0, dtype=np.complex64).ravel()
    tau_s = tf[r00] * w00 + tf[r01] * w01 + tf[r10] * w10 + tf[r11] * w11
    phi_s = pf[r00] * w00 + pf[r01] * w01 + pf[r10] * w10 + pf[r11] * w11
    E0_s = Ef[r00] * w00 + Ef[r01] * w01 + Ef[r10] * w10 + Ef[r11] * w11
    s_vals = pos[inb, 0] * khat[0] + pos[inb, 1] * khat[1] + pos[inb, 2] * khat[2]
    denom = float(s_max) - float(s_min)
    if not denom > 0.0:
        denom = 1.0
    f = np.clip((s_vals - float(s_min)) / denom, 0.0, 1.0).astype(np.float32)
    amp = np.exp(-f * tau_s).astype(np.float32)
    ph = f * phi_s
    c, sn = np.cos(ph), np.sin(ph)
    re = (E0_s.real * c - E0_s.imag * sn) * amp
    im = (E0_s.real * sn + E0_s.imag * c) * amp
    out[inb] = (re + 1j * im).astype(np.complex64)
    return out


def blur_map(m, rad):
    """The reference's optional Gaussian blur of tau and phi (Beam.py:7268-7277):
    a (2 rad + 1)^2 Gaussian of sigma rad / 2, zero-padded at the map's corner,
    applied by FFT (circular)."""
    sig = rad / 2.0
    y, x = np.ogrid[-rad:rad + 1, -rad:rad + 1]
    k = np.exp(-(x * x + y * y) / (2.0 * sig * sig)).astype(np.float32)
    k /= k.sum()
    Fk = np.fft.fft2(k, s=m.shape)
    return np.fft.ifft2(np.fft.fft2(m) * Fk).real.astype(np.float32)


def column_map(lab_A, fwd_re, fwd_im, grid_shape, du, dv, uc, vc, wavelength_A,
               e1=(0, 1, 0), e2=(0, 0, 1), kernel_radius=0):
    """Transmission map A(u, v) = exp(-tau + i phi) of the sample on the beam
    grid (Beam.py:7118-7283): each atom's forward factors f0(0) + f' and f''
    deposited with 3 x 3 triangular-shaped-cloud weights around its grid
    position, column sums -> phi = -k delta, tau = max(k beta, 0) with
    delta, beta = r_e lambda^2 / (2 pi du dv) x sums. lab_A (N, 3) float32
    Angstrom (after the stage transform); returns complex64 (NyB, NzB)."""
    NyB, NzB = grid_shape
    pos = np.asarray(lab_A, dtype=np.float32)
    e1 = np.asarray(e1, dtype=np.float64)
    e2 = np.asarray(e2, dtype=np.float64)
    sr = np.zeros((NyB, NzB), np.float32)
    si = np.zeros((NyB, NzB), np.float32)

    def tsc(d):
        w = np.zeros_like(d, dtype=np.float32)
        m0 = d <= 0.5
        w[m0] = 0.75 - d[m0] * d[m0]
        m1 = (~m0) & (d <= 1.5)
        t = 1.5 - d[m1]
        w[m1] = 0.5 * t * t
        return w

    au = pos[:, 0] * e1[0] + pos[:, 1] * e1[1] + pos[:, 2] * e1[2]
    av = pos[:, 0] * e2[0] + pos[:, 1] * e2[1] + pos[:, 2] * e2[2]
    iu = au / du + uc
    iv = av / dv + vc
    inb = (iu >= 0.0) & (iu <= NyB - 1) & (iv >= 0.0) & (iv <= NzB - 1)
    if np.any(inb):
        iu, iv = iu[inb], iv[inb]
        fr = np.asarray(fwd_re, np.float32)[inb]
        fi = np.asarray(fwd_im, np.float32)[inb]
        ic = np.floor(iu + 0.5).astype(np.int64)
        jc = np.floor(iv + 0.5).astype(np.int64)
        for dx in (-1, 0, 1):
            wx = tsc(np.abs(iu - (ic + dx)))
            for dy in (-1, 0, 1):
                wy = tsc(np.abs(iv - (jc + dy)))
                fac = wx * wy
                ii, jj = ic + dx, jc + dy
                m = (ii >= 0) & (ii < NyB) & (jj >= 0) & (jj < NzB) & (fac > 0.0)
                idx = ii[m] * NzB + jj[m]
                np.add.at(sr.ravel(), idx, (fr[m] * fac[m]).astype(np.float32))
                np.add.at(si.ravel(), idx, (fi[m] * fac[m]).astype(np.float32))
    r_e_A = 2.81794092e-5
    C = (r_e_A * wavelength_A * wavelength_A) / (2.0 * np.pi * du * dv)
    kA = 2.0 * np.pi / wavelength_A
    phi = (-kA * (C * sr)).astype(np.float32)
    tau = np.maximum((kA * (C * si)).astype(np.float32), np.float32(0.0))
    if kernel_radius > 0:
        phi = blur_map(phi, int(kernel_radius))
        tau = np.maximum(blur_map(tau, int(kernel_radius)), np.float32(0.0))
    return np.exp(-tau + 1j * phi).astype(np.complex64)


def interact_cpu(chunks, pixel_coords_A, shape, rotation, translation, energy_eV,
                 f0_rows, f0_zero, f1f2_tables, E0, beam_grid, pol_state,
                 remove_forward=False, apply_polarization=False,
                 spherical_decay=False, dw_b=None, n_threads=None, analyser=None,
                 depth=False, kernel="oracle"):
    """Restatement of ``interact_beam_cpu`` (Beam.py:5773-5956), returning
    complex128 (Nz, Ny). ``analyser`` (see ``scatter_f64``) adds the GPU
    general kernel's analyser factor, which the reference's CPU path does not
    apply. ``depth`` uses the depth-dependent incident field
    (Beam.py:4963-5140: transmission map of the whole sample, global depth
    window, ``ein_depth``) instead of E0 alone.

    chunks: iterable of (positions (N,3) float32 A, species labels (N,)).
    beam_grid: (du, dv, uc, vc). f0_rows: element -> (11,) float32;
    f0_zero: element -> float; f1f2_tables: element -> (M,3) float32.
    dw_b: None or element -> B (A^2).
    kernel: "oracle" (the FP64 C restatement) or "reference" (the
    reference's own compute_scattering_cffi, ``scatter_ref``; no
    Debye-Waller factor or analyser).
    """
    Ny, Nz = shape
    lam = H_PLANCK / Q_E * C_LIGHT / float(energy_eV)
    k = float(2.0 * np.pi / lam)
    cx, cy, cz = (np.asarray(pixel_coords_A[i]).astype(np.float64) / 1e10 for i in range(3))
    out = np.zeros(Ny * Nz, dtype=np.complex128)
    R = np.asarray(rotation, dtype=np.float32)
    T = np.asarray(translation, dtype=np.float32)
    du, dv, uc, vc = beam_grid
    tau_d = phi_d = None
    if depth:
        labs, fr_all, fi_all = [], [], []
        for pos, spc in chunks:
            pos = np.asarray(pos, dtype=np.float32)
            if pos.shape[0] == 0:
                continue
            spc = np.asarray(spc).astype(str)
            lab = (pos @ R.T + T).astype(np.float32)
            fr = np.zeros(pos.shape[0], np.float32)
            fi = np.zeros(pos.shape[0], np.float32)
            for el in np.unique(spc):
                m = spc == el
                c = anomalous(energy_eV, f1f2_tables[el]) if el in f1f2_tables else 0j
                fr[m] = np.float32(f0_zero.get(el, 0.0)) + np.float32(c.real)
                fi[m] = np.float32(c.imag)
            labs.append(lab)
            fr_all.append(fr)
            fi_all.append(fi)
        lab_all = np.concatenate(labs)
        A = column_map(lab_all, np.concatenate(fr_all), np.concatenate(fi_all), E0.shape,
                       du, dv, uc, vc, lam * 1e10)
        tau_d = (-np.log(np.abs(A) + np.float32(1e-20))).astype(np.float32)
        phi_d = np.angle(A).astype(np.float32)
        s_min, s_max = float(lab_all[:, 0].min()), float(lab_all[:, 0].max())
        if not s_max > s_min:
            s_min, s_max = 0.0, 1.0
    for pos, spc in chunks:
        pos = np.asarray(pos, dtype=np.float32)
        spc = np.asarray(spc).astype(str)
        n = pos.shape[0]
        if n == 0:
            continue
        lab = (pos @ R.T + T).astype(np.float32)
        amp = (ein_depth(lab, E0, tau_d, phi_d, du, dv, uc, vc, s_min, s_max) if depth
               else ein_bilinear(lab, E0, du, dv, uc, vc))
        wk = np.zeros((n, 11), np.float32)
        f0z = np.zeros(n, np.float32)
        ar = np.zeros(n, np.float32)
        ai = np.zeros(n, np.float32)
        b = np.zeros(n, np.float32)
        for el in np.unique(spc):
            if el not in f0_rows:
                continue
            m = spc == el
            wk[m] = f0_rows[el]
            f0z[m] = float(f0_zero[el])
            if el in f1f2_tables:
                c = anomalous(energy_eV, f1f2_tables[el])
                ar[m] = c.real
                ai[m] = c.imag
            if dw_b is not None:
                b[m] = float(dw_b.get(el, 0.0))
        if kernel == "reference":
            if dw_b is not None or analyser is not None:
                raise ValueError("the reference CPU kernel has no Debye-Waller factor or analyser")
            out += scatter_ref(lab.astype(np.float64) / 1e10, wk, f0z, ar, ai, amp.real,
                               amp.imag, cx, cy, cz, k, Ny, Nz, remove_forward=remove_forward,
                               apply_pol=apply_polarization, pol=pol_state, decay=spherical_decay,
                               n_threads=n_threads)
            continue
        out += scatter_f64(lab.astype(np.float64) / 1e10, wk, f0z, ar, ai,
                           amp.real, amp.imag, cx, cy, cz, k, Ny, Nz,
                           remove_forward=remove_forward, apply_pol=apply_polarization,
                           pol=pol_state, decay=spherical_decay,
                           dw_b=None if dw_b is None else b, n_threads=n_threads,
                           analyser=analyser)
    return out.reshape(Nz, Ny)
