"""Free-space propagation of the detector field (angular spectrum).

Follows the reference's ``_angular_spectrum_propagate_gpu`` and
``wavefield_propagation`` (Beam.py:4622-4736, 7829-8095): the field is padded
to a power-of-two grid sized for the distance, transformed, multiplied by the
exact free-space transfer function with the carrier removed, transformed
back and centre-cropped; distances the padded grid cannot sample without
aliasing are split into equal alias-free steps. Here the 2-D transform is
split by dimension: the row (y) transforms, over contiguous rows, are cuFFT
through torch.fft, and one libmosaic_kin kernel (``mk_prop_cols``) does the
column transform, the transfer-function multiply and the inverse column
transform for groups of neighbouring columns in shared memory, so the
spectrum makes one round trip through HBM between the row transforms
instead of three. The pad and the crop (fused with |A|^2) are
libmosaic_kin kernels too. ``fused=False`` runs the unfused sequence
(cuFFT 2-D transforms around ``mk_prop_mul``, FP64 phase) instead.

``FreeSpaceStack`` is a minimal optics stack with the reference's
``apply_stack`` interface holding free-space segments only (the reference's
lenses, magnifiers, filters and apertures are outside this library); a
reference ``optics`` object can be passed instead.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import engine
from ._lib import check


def next_pow_two(n) -> int:
    n = int(np.ceil(n))
    return 1 if n < 1 else 1 << (n - 1).bit_length()


def choose_optimal_pad(Ny, Nz, dy, dz, wavelength, z, safety=1.1, enforce_pow2=True,
                       min_pad_factor=1.0):
    """Padded sizes so nothing wraps after distance |z| (Beam.py:4632-4700)."""
    zabs = abs(float(z))
    if zabs == 0.0:
        Ny2 = max(int(np.ceil(Ny * min_pad_factor)), Ny)
        Nz2 = max(int(np.ceil(Nz * min_pad_factor)), Nz)
        if enforce_pow2:
            Ny2, Nz2 = next_pow_two(Ny2), next_pow_two(Nz2)
        return int(Ny2), int(Nz2)
    sry = min(min(1.0, float(wavelength) / (2.0 * float(dy))), 0.999999)
    srz = min(min(1.0, float(wavelength) / (2.0 * float(dz))), 0.999999)
    tany = min(sry / np.sqrt(max(1e-18, 1.0 - sry * sry)), 2.0)
    tanz = min(srz / np.sqrt(max(1e-18, 1.0 - srz * srz)), 2.0)
    pad_y = int(np.ceil(safety * zabs * tany / float(dy)))
    pad_z = int(np.ceil(safety * zabs * tanz / float(dz)))
    Ny2 = max(Ny + 2 * pad_y, int(np.ceil(Ny * min_pad_factor)))
    Nz2 = max(Nz + 2 * pad_z, int(np.ceil(Nz * min_pad_factor)))
    Ny2, Nz2 = min(Ny2, 8192), min(Nz2, 8192)
    if enforce_pow2:
        Ny2, Nz2 = next_pow_two(Ny2), next_pow_two(Nz2)
    return int(Ny2), int(Nz2)


def alias_free_step(Ny, Nz, dy, dz, wavelength, z, pad_factor=1.0):
    """Largest single step the padded grid samples without aliasing
    (Beam.py:4704-4736)."""
    Ny2, Nz2 = choose_optimal_pad(int(Ny), int(Nz), dy, dz, wavelength, z,
                                  min_pad_factor=max(1.0, float(pad_factor)))
    zy = Ny2 * float(dy) ** 2 / float(wavelength)
    zz = Nz2 * float(dz) ** 2 / float(wavelength)
    return float(min(zy, zz)) if (zy > 0 and zz > 0) else float("inf")


def _as_device_c64(field, device):
    if isinstance(field, torch.Tensor):
        t = field.to(device=device)
    else:
        t = torch.as_tensor(np.ascontiguousarray(field))
        t = t.to(device)
    return t.to(torch.complex64).contiguous()


def propagate(field, dy, dz, z, wavelength, step_max=None, pad_factor=1.0, padding_mode="edge",
              pad_constant=0.0, k_axis=None, k_perp_y=0.0, k_perp_z=0.0, intensity=False,
              device="cuda", fused=True):
    """Propagate a (Nz, Ny) field over z [m]. Returns the complex64 field on
    the device, or (field, |field|^2) with ``intensity``."""
    L = engine._require_cuda()
    E = _as_device_c64(field, device)
    Nz, Ny = int(E.shape[0]), int(E.shape[1])
    z = float(z)
    limit = alias_free_step(Ny, Nz, dy, dz, wavelength, z, pad_factor) if step_max is None \
        else float(step_max)
    n_steps = int(np.ceil(abs(z) / limit)) if abs(z) > limit else 1
    dz_step = z / n_steps
    k = 2.0 * np.pi / float(wavelength)
    kga = k if k_axis is None else float(k_axis)
    sh = engine._stream_handle()
    I = None
    for s in range(n_steps):
        last = s == n_steps - 1
        Ny2, Nz2 = choose_optimal_pad(Ny, Nz, dy, dz, wavelength, dz_step,
                                      min_pad_factor=max(1.0, float(pad_factor)))
        y0, z0 = (Ny2 - Ny) // 2, (Nz2 - Nz) // 2
        P = torch.empty((Nz2, Ny2), dtype=torch.complex64, device=E.device)
        mode = 1 if str(padding_mode or "edge").lower() == "constant" else 0
        c = complex(pad_constant)
        check(L.mk_prop_pad(E.data_ptr(), Ny, Nz, P.data_ptr(), Ny2, Nz2, y0, z0, mode,
                            c.real, c.imag, sh))
        if fused:
            F = torch.fft.fft(P, dim=-1).contiguous()   # rows (y); already contiguous
            ws_n = int(L.mk_prop_cols_workspace_size(Ny2, Nz2))
            ws = torch.empty(ws_n, dtype=torch.uint8, device=E.device)
            check(L.mk_prop_cols(F.data_ptr(), Ny2, Nz2, float(dy), float(dz), k, dz_step, kga,
                                 float(k_perp_y), float(k_perp_z), ws.data_ptr(), ws_n, sh))
            G = torch.fft.ifft(F, dim=-1, norm="forward")   # unnormalised; 1/N in the crop
        else:
            F = torch.fft.fft2(P)
            check(L.mk_prop_mul(F.data_ptr(), Ny2, Nz2, float(dy), float(dz), k, dz_step, kga,
                                float(k_perp_y), float(k_perp_z), sh))
            G = torch.fft.ifft2(F, norm="forward")        # unnormalised; 1/N in the crop
        out = torch.empty((Nz, Ny), dtype=torch.complex64, device=E.device)
        if intensity and last:
            I = torch.empty((Nz, Ny), dtype=torch.float32, device=E.device)
        check(L.mk_prop_crop_abs2(G.data_ptr(), Ny2, Nz2, y0, z0, Ny, Nz,
                                  1.0 / float(Ny2 * Nz2), out.data_ptr(),
                                  I.data_ptr() if I is not None else None, sh))
        E = out
    return (E, I) if intensity else E


class FreeSpaceStack:
    """Optics stack of free-space segments with the reference's apply_stack
    interface (Optics.py:513-639, 743-753)."""

    def __init__(self, lengths_mm=()):
        self.components = [{"kind": "free space", "length": float(l)} for l in lengths_mm]

    def add_free_space(self, length_mm):
        self.components.append({"kind": "free space", "length": float(length_mm)})

    def apply_stack(self, field, dx, dy, wavelength, propagate_free_space, use_gpu=True,
                    diagnostics=False):
        E = field
        for elem in self.components:
            if str(elem.get("kind", "")).lower() != "free space":
                raise NotImplementedError(f"optics component '{elem.get('kind')}' is not provided")
            E = propagate_free_space(E, dx, dy, float(elem.get("length", 0.0)) * 1e-3)
        return E
