"""The C-ABI library builds, loads, and exports every entry point that
include/mosaic_kin.h declares; argument checks that run before any CUDA call
return their status codes without a GPU."""
import ctypes
import os
import re

import pytest

from mosaic_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "mosaic_kin.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(mk_[a-z_0-9]+)\s*\(", src,
                                 flags=re.M)))


def test_header_declares_the_entry_points():
    fns = declared_functions()
    assert {"mk_version", "mk_last_error", "mk_sync_status", "mk_kin_plain_f64",
            "mk_kin_split_f32", "mk_tiles_build", "mk_pixels_prepare"} <= set(fns)


def test_library_builds_and_exports_every_declared_symbol():
    so = _lib.build()
    assert os.path.exists(so)
    L = ctypes.CDLL(so)
    for name in declared_functions():
        assert hasattr(L, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"


def test_version_and_host_side_validation():
    L = _lib.load()
    assert L.mk_version() >= 10000
    # null arguments are rejected before any CUDA call
    assert L.mk_pixels_prepare(None, None, None) == _lib.MK_EINVAL
    assert b"null" in L.mk_last_error()
    assert L.mk_kin_split_f32(None, None, None, None, None, None, 0, None, 0, None) == _lib.MK_EINVAL
    assert L.mk_kin_plain_f64(0, None, None, None, None, None, None, 0, None, 0, None, 0,
                              None) == _lib.MK_EINVAL
    assert L.mk_sum_workspace_size(1000, 3) == 1000 * 3 * 16
    # the factor table: no buffer, or remove_forward (whose Q < Q_cut test
    # stays per tile and pixel), refused before any CUDA call
    assert L.mk_factor_table(None, None, None, 1, None, None) == _lib.MK_EINVAL
    buf = ctypes.c_void_p(256)
    px = _lib.MkPixels(4, 4, buf, buf, buf, buf, buf)
    sp = _lib.MkSpecies(1, buf, buf, buf, buf, None)
    ph = _lib.MkPhysics()
    ph.k = 5.0e10
    assert L.mk_factor_table(ctypes.byref(px), ctypes.byref(sp), ctypes.byref(ph), 1, None,
                             None) == _lib.MK_EINVAL
    assert b"factor buffer" in L.mk_last_error()
    px.factor = buf
    ph.remove_forward = 1
    assert L.mk_factor_table(ctypes.byref(px), ctypes.byref(sp), ctypes.byref(ph), 1, None,
                             None) == _lib.MK_EINVAL
    assert b"remove_forward" in L.mk_last_error()
    ph.remove_forward = 0
    assert L.mk_factor_table(ctypes.byref(px), ctypes.byref(sp), ctypes.byref(ph), 3, None,
                             None) == _lib.MK_EINVAL
    assert b"frame table" in L.mk_last_error()
    with pytest.raises(ValueError):
        _lib.check(_lib.MK_EINVAL)
    with pytest.raises(MemoryError):
        _lib.check(_lib.MK_ENOMEM)
    with pytest.raises(_lib.DeclineError):
        _lib.check(_lib.MK_EDECLINE)


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of the C structs have the header's size and field
    offsets (compiled with the host C compiler)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    structs = {"mk_species": _lib.MkSpecies, "mk_physics": _lib.MkPhysics,
               "mk_pixels": _lib.MkPixels, "mk_frame_desc": _lib.MkFrameDesc,
               "mk_tiles": _lib.MkTiles, "mk_launch": _lib.MkLaunch}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "mosaic_kin.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_scan_plan_checks_quad_rows_before_any_cuda_call():
    """Pixel quads need every frame's row length, and whole rows; octets
    need whole 2x4 octets, squares whole 4x4 squares; an unknown pixel mode
    is refused: all argument
    errors from mk_scan_plan, raised before it touches the GPU."""
    L = _lib.load()
    tiles = _lib.MkTiles(4, 128, None, None, None, None)
    launch = _lib.MkLaunch(8, 128, 0, 1, 1, 0.0, 2, 0.0, 0.0)
    npix = (ctypes.c_int * 2)(16, 12)
    bdir = (ctypes.c_double * 6)(1, 0, 0, 1, 0, 0)
    desc = (_lib.MkFrameDesc * 2)()
    ni, npart = ctypes.c_longlong(0), ctypes.c_longlong(0)

    def plan(rows):
        return L.mk_scan_plan(2, ctypes.cast(npix, ctypes.c_void_p), rows,
                              ctypes.cast(bdir, ctypes.c_void_p), None, ctypes.byref(tiles),
                              ctypes.byref(launch), ctypes.cast(desc, ctypes.c_void_p),
                              ctypes.byref(ni), ctypes.byref(npart))
    assert plan(None) == _lib.MK_EINVAL
    assert b"row length" in L.mk_last_error()
    bad = (ctypes.c_int * 2)(4, 5)          # 12 pixels are not rows of 5
    assert plan(ctypes.cast(bad, ctypes.c_void_p)) == _lib.MK_EINVAL
    assert b"whole rows" in L.mk_last_error()
    launch.pairs = 3
    assert plan(ctypes.cast(bad, ctypes.c_void_p)) == _lib.MK_EINVAL
    assert b"whole rows" in L.mk_last_error()
    odd = (ctypes.c_int * 2)(4, 6)          # 16 = 4 x 4 octets, but 12 = 2 rows of 6
    assert plan(ctypes.cast(odd, ctypes.c_void_p)) == _lib.MK_EINVAL
    assert b"octets" in L.mk_last_error()
    launch.pairs = 4
    launch.pix_per_thread = 16
    assert plan(ctypes.cast(odd, ctypes.c_void_p)) == _lib.MK_EINVAL   # 16 = 4 rows of 4: ok;
    assert b"squares" in L.mk_last_error()                             # 12 = 2 rows of 6: not
    sq_ok_first = (ctypes.c_int * 2)(4, 4)
    npix[1] = 8                                                        # 8 = 2 rows of 4
    assert plan(ctypes.cast(sq_ok_first, ctypes.c_void_p)) == _lib.MK_EINVAL
    assert b"squares" in L.mk_last_error()
    launch.pairs = 5
    assert plan(ctypes.cast(bad, ctypes.c_void_p)) == _lib.MK_EINVAL
    assert b"pairs must be" in L.mk_last_error()


def test_noalloc_scratch_size_matches_the_header():
    src = open(HEADER).read()
    m = re.search(r"#define\s+MK_NOALLOC_SCRATCH_BYTES\s+\((\d+)u\s*<<\s*(\d+)\)", src)
    assert m, "MK_NOALLOC_SCRATCH_BYTES not found"
    assert int(m.group(1)) << int(m.group(2)) == _lib.MK_NOALLOC_SCRATCH_BYTES
