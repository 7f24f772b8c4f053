"""Recipe: the reference's own scattering kernels, built from their source.

TEST INFRASTRUCTURE ONLY -- nothing in ``mosaic_gb300`` imports this module.

MOSAIC keeps its CPU kernel ``compute_scattering_cffi`` as a C source string
inside ``Beam.py`` (``beam.compile_compute_scattering_cffi``, Beam.py:621-817)
and compiles it with cffi at run time. This recipe reads that string out of
a reference checkout and writes it, unchanged, to ``oracle/_ref/ref_scatter.c``
(git-ignored: the reference's source never enters this repository), then
compiles it with gcc into ``oracle/_ref/libref_scatter.so``. The reference
builds it ``-O3 -march=native``; here it is ``-O3`` (the same code on x86 and
Arm hosts; the kernel is bound by its libm calls, which neither flag
vectorises).

The reference's GPU general kernel ``interaction_kernal`` (CUDA source string
of ``beam.build_interaction_kernel``, Beam.py:1698-2415) is extracted the
same way to ``oracle/_ref/ref_general.cu`` and compiled by nvcc for sm_103a
into ``oracle/_ref/libref_general_<mode>.so``, one library per compile-time
series setting (the reference compiles it with NVRTC at run time, keyed on
the same defines, Beam.py:2419-2433), each wrapped by the project's own
launcher ``oracle/ref_gpu_harness.cu`` -- a test-only comparator: the
kernel the reference runs on a GPU, run here on the GB300.

The extracted sources travel with the working tree to a machine without the
reference checkout, where ``build()`` compiles them again for that host.

    python oracle/ref_build.py /root/reference      # extract and build
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SRC = os.path.join(REF_DIR, "ref_scatter.c")
SO = os.path.join(REF_DIR, "libref_scatter.so")
DEFAULT_REFERENCE = "/root/reference"


def extract(reference_dir: str) -> str:
    """Copy the C source of compute_scattering_cffi out of Beam.py into
    oracle/_ref/ref_scatter.c; returns its path."""
    path = os.path.join(reference_dir, "Beam.py")
    with open(path, encoding="utf-8") as fh:
        text = fh.read()
    i = text.index("def compile_compute_scattering_cffi")
    a = text.index('c_source = r"""', i) + len('c_source = r"""')
    b = text.index('"""', a)
    body = text[a:b]
    if "int compute_scattering_cffi(" not in body:
        raise RuntimeError(f"{path}: compute_scattering_cffi source not found")
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = SRC + f".tmp{os.getpid()}"
    with open(tmp, "w", encoding="utf-8") as fh:
        fh.write("/* extracted unchanged from the reference's Beam.py "
                 "(compile_compute_scattering_cffi) by oracle/ref_build.py */\n")
        fh.write(body)
    os.replace(tmp, SRC)
    return SRC


GPU_SRC = os.path.join(REF_DIR, "ref_general.cu")
HARNESS = os.path.join(HERE, "ref_gpu_harness.cu")
# compile-time series settings built: series with N terms, and the exact form
GPU_MODES = ("s1", "s2", "s3", "s4", "s6", "exact")


def gpu_so(mode: str) -> str:
    return os.path.join(REF_DIR, f"libref_general_{mode}.so")


def extract_gpu(reference_dir: str) -> str:
    """Copy the CUDA source of interaction_kernal out of Beam.py into
    oracle/_ref/ref_general.cu; returns its path."""
    path = os.path.join(reference_dir, "Beam.py")
    with open(path, encoding="utf-8") as fh:
        text = fh.read()
    i = text.index("def build_interaction_kernel")
    a = text.index("_cuda_source = r'''", i) + len("_cuda_source = r'''")
    b = text.index("''';", a)
    body = text[a:b]
    if "void interaction_kernal(" not in body:
        raise RuntimeError(f"{path}: interaction_kernal source not found")
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = GPU_SRC + f".tmp{os.getpid()}"
    with open(tmp, "w", encoding="utf-8") as fh:
        fh.write("/* extracted unchanged from the reference's Beam.py "
                 "(build_interaction_kernel) by oracle/ref_build.py */\n")
        fh.write(body)
    os.replace(tmp, GPU_SRC)
    return GPU_SRC


def _mode_defines(mode: str):
    if mode == "exact":
        return ["-DGLOBAL_USE_SERIES=0", "-DN_SERIES=1"]
    return ["-DGLOBAL_USE_SERIES=1", f"-DN_SERIES={int(mode[1:])}"]


def build_gpu(reference_dir: str | None = None, force: bool = False, modes=GPU_MODES):
    """Extract (when a checkout is present) and compile the reference's GPU
    general kernel with the launcher, one .so per series setting; returns
    {mode: path} of those built (empty without the source or nvcc)."""
    import shutil
    from concurrent.futures import ThreadPoolExecutor
    ref = reference_dir or os.environ.get("MOSAIC_REFERENCE_DIR") or DEFAULT_REFERENCE
    if os.path.exists(os.path.join(ref, "Beam.py")) and (force or not os.path.exists(GPU_SRC)):
        extract_gpu(ref)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(GPU_SRC) or not os.path.exists(nvcc):
        return {}
    newest = max(os.path.getmtime(GPU_SRC), os.path.getmtime(HARNESS))

    def one(mode):
        so = gpu_so(mode)
        if not force and os.path.exists(so) and os.path.getmtime(so) >= newest:
            return mode, so
        tmp = so + f".tmp{os.getpid()}"
        # the reference's own NVRTC defines (Beam.py:2419-2433): one beam
        # channel, 128-atom chunks, exact prologue, no stage C, polarization
        # from the launch argument (the unroll factor, 4, is set in the
        # launcher)
        cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-shared",
               "-Xcompiler", "-fPIC", "-std=c++17", "-diag-suppress", "550", "-I", HERE,
               *_mode_defines(mode),
               "-DM_BEAMS_COMPILE=1", "-DCHUNK_SIZE=128", "-DN_PRO=8",
               "-DPROLOGUE_MODE=1", "-DSTAGE_C=0", "-DPOL_EXPLICIT=0", HARNESS, "-o", tmp]
        subprocess.check_call(cmd)
        os.replace(tmp, so)
        return mode, so

    with ThreadPoolExecutor(max_workers=len(modes)) as ex:
        return dict(ex.map(one, modes))


def build(reference_dir: str | None = None, force: bool = False) -> str | None:
    """Extract (when a reference checkout is present) and compile the
    reference kernel; returns the .so path, or None when neither the
    checkout nor an extracted source is available."""
    ref = reference_dir or os.environ.get("MOSAIC_REFERENCE_DIR") or DEFAULT_REFERENCE
    if os.path.exists(os.path.join(ref, "Beam.py")):
        if force or not os.path.exists(SRC):
            extract(ref)
    if not os.path.exists(SRC):
        return None
    if not force and os.path.exists(SO) and os.path.getmtime(SO) >= os.path.getmtime(SRC):
        return SO
    tmp = SO + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O3", "-shared", "-fPIC", SRC, "-o", tmp, "-lm"])
    os.replace(tmp, SO)
    return SO


if __name__ == "__main__":
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else None
    print(build(ref_dir, force=True))
    print(build_gpu(ref_dir, force=True))
