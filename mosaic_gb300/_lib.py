"""Build and load libmosaic_kin.so (the sm_103a C-ABI library) via ctypes.

The library is built in-tree from ``mosaic_gb300/csrc/*.cu`` by nvcc for
``sm_103a`` only. There is no CPU fallback: if the library cannot be built or
loaded, every GPU entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
SO = os.path.join(HERE, "libmosaic_kin.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
              "--expt-relaxed-constexpr"]
# Per-source extra flags. The FP64 plain sum must not contract a*b+c into FMA:
# it restates the uncontracted CPU arithmetic term for term.
EXTRA = {"mk_sum_f64.cu": ["--fmad=false"], "mk_depth.cu": ["--fmad=false"]}

MK_OK, MK_EINVAL, MK_ENOMEM, MK_ETIMEOUT, MK_EDECLINE, MK_ECUDA = 0, -1, -2, -3, -4, -5
MAX_SPECIES = 16
# fixed scratch of mk_kin_split_f32_noalloc (include/mosaic_kin.h)
MK_NOALLOC_SCRATCH_BYTES = 32 << 20

_lock = threading.Lock()
_lib = None


class MosaicError(RuntimeError):
    """A libmosaic_kin call returned an error status."""

    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class DeclineError(MosaicError):
    pass


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh"))]
    files.append(os.path.join(INCLUDE, "mosaic_kin.h"))
    return files


def nvcc_path():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    return cand if os.path.exists(cand) else None


def is_stale() -> bool:
    if not os.path.exists(SO):
        return True
    t = os.path.getmtime(SO)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every .cu under csrc/ for sm_103a (in parallel) and link the .so."""
    with _lock:
        if not force and not is_stale():
            return SO
        nvcc = nvcc_path()
        if nvcc is None:
            raise RuntimeError("nvcc not found: libmosaic_kin.so cannot be built")
        os.makedirs(BUILD, exist_ok=True)

        def compile_one(src):
            obj = os.path.join(BUILD, src.replace(".cu", ".o"))
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, *EXTRA.get(src, []), "-I", INCLUDE, "-c",
                   os.path.join(CSRC, src), "-o", obj]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr[-4000:]}")
            if verbose and r.stderr:
                print(r.stderr)
            return obj

        srcs = _sources()
        with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
            objs = list(ex.map(compile_one, srcs))
        tmp = SO + f".tmp{os.getpid()}"
        r = subprocess.run([nvcc, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
        os.replace(tmp, SO)
        return SO


# ------------------------------------------------------------ ABI structs
_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p


class MkSpecies(ctypes.Structure):
    _fields_ = [("n_species", ctypes.c_int), ("wk", _vp), ("f0_zero", _vp), ("anom_re", _vp),
                ("anom_im", _vp), ("dw_b", _vp)]


class MkPhysics(ctypes.Structure):
    _fields_ = [("k", ctypes.c_double), ("beam_dir", ctypes.c_double * 3),
                ("apply_pol", ctypes.c_int), ("pol_deg", ctypes.c_double),
                ("pol_e", ctypes.c_double * 3), ("spherical_decay", ctypes.c_int),
                ("remove_forward", ctypes.c_int), ("analyser", ctypes.c_int),
                ("analyser_dir", ctypes.c_double * 3), ("analyser_accept", ctypes.c_double),
                ("analyser_halfwidth", ctypes.c_double)]


class MkPixels(ctypes.Structure):
    _fields_ = [("ny", ctypes.c_int), ("nz", ctypes.c_int), ("xyz", _vp), ("r0", _vp),
                ("q", _vp), ("u", _vp), ("phasor", _vp), ("factor", _vp)]


class MkFrameDesc(ctypes.Structure):
    _fields_ = [("pix_off", ctypes.c_longlong), ("part_off", ctypes.c_longlong),
                ("item_off", ctypes.c_longlong), ("n_pix", ctypes.c_int), ("slices", ctypes.c_int),
                ("tiles_per_slice", ctypes.c_int), ("pix_blocks", ctypes.c_int),
                ("b", ctypes.c_float * 3), ("e", ctypes.c_float * 3), ("row", ctypes.c_int),
                ("reserved", ctypes.c_int * 3)]


class MkTiles(ctypes.Structure):
    _fields_ = [("n_tiles", ctypes.c_int), ("tile_atoms", ctypes.c_int), ("origin", _vp),
                ("species", _vp), ("pos", _vp), ("amp", _vp)]


class MkLaunch(ctypes.Structure):
    _fields_ = [("pix_per_thread", ctypes.c_int), ("threads", ctypes.c_int),
                ("slices", ctypes.c_int), ("fresnel", ctypes.c_int), ("amp_real", ctypes.c_int),
                ("fresnel_radius_m", ctypes.c_double), ("pairs", ctypes.c_int),
                ("pair_short_radius_m", ctypes.c_double), ("sin_direct_max_rad", ctypes.c_double),
                ("octet_radius_m", ctypes.c_double)]


# name -> (restype, argtypes)
SIGNATURES = {
    "mk_version": (ctypes.c_int, []),
    "mk_last_error": (ctypes.c_char_p, []),
    "mk_sync_status": (ctypes.c_int, [_vp]),
    "mk_pixels_prepare": (ctypes.c_int, [ctypes.POINTER(MkPixels), ctypes.POINTER(MkPhysics), _vp]),
    "mk_factor_table": (ctypes.c_int, [ctypes.POINTER(MkPixels), ctypes.POINTER(MkSpecies),
                                       ctypes.POINTER(MkPhysics), ctypes.c_int, _vp, _vp]),
    "mk_atoms_lab": (ctypes.c_int, [ctypes.c_int64, _vp, _fp, _fp, _vp, ctypes.c_int, ctypes.c_int,
                                    _dp, _vp, _vp, _vp]),
    "mk_tiles_workspace_size": (ctypes.c_size_t, [ctypes.c_int64]),
    "mk_tiles_build": (ctypes.c_int, [ctypes.c_int64, _vp, _vp, _vp, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_int64), ctypes.c_double,
                                      ctypes.POINTER(MkTiles), _vp, ctypes.c_size_t, _vp]),
    "mk_sum_workspace_size": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int]),
    "mk_kin_plain_f64": (ctypes.c_int, [ctypes.c_int64, _vp, _vp, _vp, ctypes.POINTER(MkSpecies),
                                        ctypes.POINTER(MkPhysics), ctypes.POINTER(MkPixels),
                                        ctypes.c_int, _vp, ctypes.c_int, _vp, ctypes.c_size_t, _vp]),
    "mk_debug_wait_timeout": (ctypes.c_int, [ctypes.c_uint64, _vp]),
    "mk_probe_workspace_size": (ctypes.c_size_t, []),
    "mk_probe_throughput": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _vp, ctypes.c_size_t,
                                           ctypes.POINTER(ctypes.c_double), _vp]),
    "mk_gemm_bf16": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_longlong,
                                    ctypes.c_longlong, _vp, ctypes.c_longlong, ctypes.c_longlong,
                                    _vp, ctypes.c_longlong, _vp, ctypes.c_int, _vp,
                                    ctypes.c_longlong, _vp]),
    "mk_gemm_tc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_longlong,
                                  ctypes.c_longlong, _vp, ctypes.c_longlong, ctypes.c_longlong,
                                  _vp, ctypes.c_longlong, _vp, ctypes.c_int, _vp,
                                  ctypes.c_longlong, _vp, ctypes.c_longlong, _vp, _vp, _vp]),
    "mk_gemm_tc_groups": (ctypes.c_int, [ctypes.c_int, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         _vp, ctypes.c_longlong, ctypes.c_longlong, _vp,
                                         ctypes.c_longlong, ctypes.c_longlong, _vp,
                                         ctypes.c_longlong, _vp, ctypes.c_int, _vp,
                                         ctypes.c_longlong, _vp, ctypes.c_longlong, _vp, _vp, _vp]),
    "mk_bias_grad_groups": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp,
                                           ctypes.c_longlong, _vp, ctypes.c_longlong, _vp]),
    "mk_fourier_features": (ctypes.c_int, [ctypes.c_int, _vp, ctypes.c_int, ctypes.c_float,
                                           ctypes.c_float, ctypes.c_int, _vp, _vp]),
    "mk_relu_backward": (ctypes.c_int, [ctypes.c_longlong, _vp, _vp, _vp, _vp, _vp]),
    "mk_bias_grad": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _vp, _vp, _vp]),
    "mk_beam_column_sums": (ctypes.c_int, [ctypes.c_int64, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, _vp, _vp, _vp, _vp]),
    "mk_beam_column_maps": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, _vp, _vp, _vp]),
    "mk_beam_column_wrap": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _vp, _vp, _vp]),
    "mk_atoms_ein_depth": (ctypes.c_int, [ctypes.c_int64, _vp, _vp, _vp, _vp, ctypes.c_int,
                                          ctypes.c_int, _vp, ctypes.c_double, ctypes.c_double, _vp,
                                          _vp]),
    "mk_mse": (ctypes.c_int, [ctypes.c_longlong, _vp, _vp, _vp, _vp, _vp, _vp]),
    "mk_mse_weighted": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_int, _vp, _vp, _vp, _vp, _vp,
                                       _vp, _vp]),
    "mk_adam_sched": (ctypes.c_int, [ctypes.c_longlong, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                     ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_float, _vp]),
    "mk_counter_add": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "mk_adam": (ctypes.c_int, [ctypes.c_longlong, _vp, _vp, _vp, _vp, _vp, ctypes.c_float,
                               ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_int,
                               ctypes.c_float, _vp]),
    "mk_prop_pad": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                   ctypes.c_float, _vp]),
    "mk_prop_mul": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, _vp]),
    "mk_tc_gemm": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp]),
    "mk_prop_cols": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, _vp, ctypes.c_size_t, _vp]),
    "mk_prop_cols_workspace_size": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int]),
    "mk_prop_crop_abs2": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_float, _vp, _vp, _vp]),
    "mk_split_plan": (ctypes.c_int, [ctypes.POINTER(MkTiles), ctypes.POINTER(MkPixels),
                                     ctypes.POINTER(MkLaunch), ctypes.POINTER(ctypes.c_size_t)]),
    "mk_kin_split_f32_noalloc": (ctypes.c_int, [ctypes.POINTER(MkTiles), ctypes.POINTER(MkSpecies),
                                                ctypes.POINTER(MkPhysics), ctypes.POINTER(MkPixels),
                                                ctypes.POINTER(MkLaunch), _vp, ctypes.c_int, _vp]),
    "mk_scan_plan": (ctypes.c_int, [ctypes.c_int, _vp, _vp, _vp, _vp, ctypes.POINTER(MkTiles),
                                    ctypes.POINTER(MkLaunch), _vp, ctypes.POINTER(ctypes.c_longlong),
                                    ctypes.POINTER(ctypes.c_longlong)]),
    "mk_scan_workspace_size": (ctypes.c_size_t, [ctypes.c_longlong]),
    "mk_kin_scan_f32": (ctypes.c_int, [ctypes.POINTER(MkTiles), ctypes.POINTER(MkSpecies),
                                       ctypes.POINTER(MkPhysics), ctypes.POINTER(MkPixels),
                                       ctypes.c_int, _vp, ctypes.c_longlong, ctypes.c_longlong,
                                       ctypes.POINTER(MkLaunch), _vp, _vp, _vp, ctypes.c_size_t, _vp]),
    "mk_kin_split_f32": (ctypes.c_int, [ctypes.POINTER(MkTiles), ctypes.POINTER(MkSpecies),
                                        ctypes.POINTER(MkPhysics), ctypes.POINTER(MkPixels),
                                        ctypes.POINTER(MkLaunch), _vp, ctypes.c_int, _vp,
                                        ctypes.c_size_t, _vp]),
}


def load(build_if_needed: bool = True):
    """The loaded library (built first when stale). Raises if unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_needed and is_stale():
        build()
    if not os.path.exists(SO):
        raise RuntimeError(f"{SO} is missing; run mosaic_gb300._lib.build()")
    L = ctypes.CDLL(SO)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc: int) -> None:
    """Raise MosaicError (DeclineError for MK_EDECLINE) on a non-zero status."""
    if rc == MK_OK:
        return
    msg = (load().mk_last_error() or b"").decode(errors="replace")
    if rc == MK_EDECLINE:
        raise DeclineError(rc, msg)
    if rc == MK_ENOMEM:
        raise MemoryError(msg)
    if rc == MK_EINVAL:
        raise ValueError(msg)
    raise MosaicError(rc, msg)
