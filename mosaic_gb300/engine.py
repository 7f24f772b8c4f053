"""Device-side staging and launches for the kinematic sum.

PyTorch supplies device memory and the stream; every computation on the
path runs in libmosaic_kin.so (``include/mosaic_kin.h``) through ctypes.

Data layout in HBM (one GPU):
  atoms    pos_lab float64 (N, 3) [m], species int32 (N), amp float32 (N, 2)
  tiles    origin float64 (n_tiles, 4) [m], species int32 (n_tiles),
           pos float32 (n_tiles*T, 4) = k/2pi (a - o) [cycles] and its |.|^2,
           amp float32 (n_tiles*T, 2); each species run padded to whole tiles
  pixels   xyz float64 (3, P) [m] and the derived r0, qcut, qc, uf, phasor
  output   complex128 (P,) = float64 (P, 2)
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from ._lib import MkLaunch, MkPhysics, MkPixels, MkSpecies, MkTiles, check

R_E = 2.81794092e-15


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("mosaic_gb300 needs a CUDA GPU: there is no CPU path")
    return _lib.load()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _stream_handle(stream=None):
    s = stream or torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


# Atoms per tile when nothing is tuned: 512, where the 4x4 square form runs
# the 8.19M-atom exposure fastest (6,693 Gatom*px/s against 6,426 on 1024-atom
# tiles and 5,687 for octets on 1024); the other forms lose ~2 % against 1024.
DEFAULT_TILE_ATOMS = 512

@dataclass
class SpeciesTable:
    """Per-species arrays in kernel order (host float32)."""
    labels: list
    wk: np.ndarray
    f0z: np.ndarray
    anom: np.ndarray
    dw_b: np.ndarray | None = None

    @classmethod
    def build(cls, labels, tables, energy_eV, dw_b=None):
        labels = [str(x) for x in labels]
        if len(labels) > _lib.MAX_SPECIES:
            raise ValueError(f"at most {_lib.MAX_SPECIES} species per call, got {len(labels)}")
        wk = np.stack([tables.row(e) for e in labels]).astype(np.float32)
        f0z = np.array([tables.f0_zero(e) for e in labels], dtype=np.float32)
        an = np.array([tables.anomalous(e, energy_eV) for e in labels], dtype=np.complex128)
        b = None
        if dw_b is not None:
            b = np.array([float(dw_b.get(e, 0.0)) for e in labels], dtype=np.float32)
            if not np.any(b):
                b = None
        return cls(labels, wk, f0z, an, b)

    def key(self):
        """What the factor of each species depends on (labels, f0
        coefficients, f(0), f' + i f'', Debye-Waller B)."""
        dw = b"" if self.dw_b is None else np.asarray(self.dw_b, np.float32).tobytes()
        return (tuple(self.labels), np.asarray(self.wk, np.float32).tobytes(),
                np.asarray(self.f0z, np.float32).tobytes(),
                np.asarray(self.anom, np.complex128).tobytes(), dw)

    def abi(self):
        self._keep = [np.ascontiguousarray(self.wk, np.float32),
                      np.ascontiguousarray(self.f0z, np.float32),
                      np.ascontiguousarray(self.anom.real, np.float32),
                      np.ascontiguousarray(self.anom.imag, np.float32),
                      None if self.dw_b is None else np.ascontiguousarray(self.dw_b, np.float32)]
        w, z, ar, ai, b = self._keep
        return MkSpecies(len(self.labels), w.ctypes.data, z.ctypes.data, ar.ctypes.data,
                         ai.ctypes.data, None if b is None else b.ctypes.data)


ANALYSER_KINDS = {"off": 0, "none": 0, "disabled": 0, "top_hat": 1, "tophat": 1, "top-hat": 1,
                  "top": 1, "darwin": 2, "rolloff": 2, "roll-off": 2}


# (threads, pixels per thread) the split kernel's analyser variant is built for
ANALYSER_LAUNCHES = ((128, 2), (128, 4), (256, 2), (256, 4))


def analyser_kind(mode):
    """Analyser mode (name or 0/1/2) -> 0 off, 1 top-hat, 2 Darwin; unknown
    names and codes mean off, as in the reference (Beam.py:6134-6143)."""
    if mode is None:
        return 0
    if isinstance(mode, str):
        return ANALYSER_KINDS.get(mode.strip().lower(), 0)
    k = int(mode)
    return k if k in (1, 2) else 0


def physics(k, beam_dir=(1.0, 0.0, 0.0), apply_pol=False, pol=(0.0, 0.0, 1.0, 0.0),
            spherical_decay=False, remove_forward=False, analyser=None):
    """mk_physics. ``analyser`` = (kind, axis (3,), acceptance [rad],
    Darwin half-width [rad]) or None."""
    ph = MkPhysics()
    ph.k = float(k)
    ph.beam_dir[:] = [float(v) for v in beam_dir]
    ph.apply_pol = int(bool(apply_pol))
    ph.pol_deg = float(pol[0])
    ph.pol_e[:] = [float(v) for v in pol[1:4]]
    ph.spherical_decay = int(bool(spherical_decay))
    ph.remove_forward = int(bool(remove_forward))
    if analyser is not None and analyser_kind(analyser[0]):
        axis = np.asarray(analyser[1], dtype=np.float64).reshape(3)
        nrm = float(np.linalg.norm(axis))
        if not nrm > 0.0:
            raise ValueError("analyser axis must be a non-zero vector")
        ph.analyser = analyser_kind(analyser[0])
        ph.analyser_dir[:] = [float(v) for v in axis / nrm]
        ph.analyser_accept = float(analyser[2])
        ph.analyser_halfwidth = float(analyser[3])
    return ph


class Pixels:
    """Detector pixels on the device plus their per-pixel prologue.

    ``xyz_m`` is (3, P) in metres (the detector's layout), host or device.
    With ``frames`` (a list of (ny, nz, beam_dir) per frame whose pixels are
    consecutive in xyz_m) every frame's prologue uses its own direction."""

    def __init__(self, xyz_m, ny, nz, phys, device="cuda", stream=None, frames=None):
        L = _require_cuda()
        P = int(ny) * int(nz)
        if isinstance(xyz_m, torch.Tensor):
            x = xyz_m.to(device=device, dtype=torch.float64).reshape(3, P)
        else:
            x = torch.as_tensor(np.ascontiguousarray(xyz_m, dtype=np.float64).reshape(3, P)).to(device)
        self.xyz = x.t().contiguous()                    # (P, 3)
        dd = dict(dtype=torch.float64, device=device)
        self.r0 = torch.empty(P, **dd)
        self.q = torch.empty((P, 4), **dd)
        self.u = torch.empty((P, 4), dtype=torch.float32, device=device)
        self.phasor = torch.empty((P, 2), **dd)
        self.ny, self.nz, self.n = int(ny), int(nz), P
        self.abi = MkPixels(self.ny, self.nz, self.xyz.data_ptr(), self.r0.data_ptr(),
                            self.q.data_ptr(), self.u.data_ptr(), self.phasor.data_ptr())
        sh = _stream_handle(stream)
        self.spans = [(0, P)]
        self.shapes = [(self.ny, self.nz)]
        if frames is None:
            check(L.mk_pixels_prepare(ctypes.byref(self.abi), ctypes.byref(phys), sh))
            return
        off = 0
        self.spans = []
        self.shapes = [(int(fny), int(fnz)) for fny, fnz, _ in frames]
        for fny, fnz, bdir in frames:
            m = int(fny) * int(fnz)
            sub = MkPixels(int(fny), int(fnz), self.xyz[off:].data_ptr(), self.r0[off:].data_ptr(),
                           self.q[off:].data_ptr(), self.u[off:].data_ptr(),
                           self.phasor[off:].data_ptr())
            ph = MkPhysics.from_buffer_copy(phys)
            ph.beam_dir[:] = [float(v) for v in bdir]
            check(L.mk_pixels_prepare(ctypes.byref(sub), ctypes.byref(ph), sh))
            self.spans.append((off, m))
            off += m
        if off != P:
            raise ValueError(f"frames cover {off} pixels, xyz has {P}")

    def factor_table(self, table, phys, stream=None):
        """(n_species, P, 2) float32 scattering factors of every species at
        every pixel's own direction (``mk_factor_table``), for single
        exposures (the physics' beam direction); kept per Pixels object for
        the last species table and physics it was made for."""
        key = (table.key(), float(phys.k), tuple(phys.beam_dir), int(phys.apply_pol),
               float(phys.pol_deg), tuple(phys.pol_e))
        cached = getattr(self, "_ftab", None)
        if cached is not None and cached[0] == key:
            return cached[1]
        L = _require_cuda()
        ftab = torch.empty((len(table.labels), self.n, 2), dtype=torch.float32,
                           device=self.xyz.device)
        abi = MkPixels.from_buffer_copy(self.abi)
        abi.factor = ftab.data_ptr()
        sp = table.abi()
        check(L.mk_factor_table(ctypes.byref(abi), ctypes.byref(sp), ctypes.byref(phys), 1, None,
                                _stream_handle(stream)))
        self._ftab = (key, ftab)
        return ftab

    def r0_min(self):
        """Smallest pixel distance (one read-back per Pixels object)."""
        if getattr(self, "_r0_min", None) is None:
            self._r0_min = float(self.r0.min())
        return self._r0_min

    def pair_step(self):
        """Largest |u_2j - u_2j+1| over the pixel pairs (2j, 2j+1) of every
        frame, u the unit vector to the pixel: the pairs mode shares one
        sin/cos between the two pixels of a pair (once per Pixels object)."""
        if getattr(self, "_pair_step", None) is not None:
            return self._pair_step
        u = self.u[:, :3].double()
        worst = 0.0
        if all(off % 2 == 0 for off, _ in self.spans):
            h = self.n // 2
            if h:
                worst = float(torch.linalg.vector_norm(u[0:2 * h:2] - u[1:2 * h:2], dim=1).max())
        else:
            for off, m in self.spans:
                h = m // 2
                if h:
                    d = u[off:off + 2 * h:2] - u[off + 1:off + 2 * h:2]
                    worst = max(worst, float(torch.linalg.vector_norm(d, dim=1).max()))
        self._pair_step = worst
        return worst

    def row_lengths(self):
        """Pixels per detector row of every frame (the kernel's quad layout)."""
        return [ny for ny, _ in self.shapes]

    def quad_steps(self):
        """Differences of the FP64 unit vectors u to the pixels over the 2x2
        quads (a b / c d: a, b neighbours in a row, c, d below them) of every
        frame, laid out as the kernel does: an odd last column or row repeats
        its pixels (the quad's difference across it is then 0). Returns the
        largest norms of the row difference (b - a) + (d - c), the cross-row
        difference (c - a) + (d - b), the mixed difference (a - b) + (d - c)
        and the diagonals d - a, c - b (computed once per Pixels object)."""
        if getattr(self, "_quad_steps", None) is not None:
            return dict(self._quad_steps)
        x = self.xyz
        u = x / torch.linalg.vector_norm(x, dim=1, keepdim=True)
        # frames of one shape at once (a scan has few distinct ROI shapes);
        # one read-back at the end
        groups = {}
        for (off, m), shp in zip(self.spans, self.shapes):
            groups.setdefault(shp, []).append(off)
        parts = []
        nrm = lambda t: torch.linalg.vector_norm(t, dim=-1).amax()
        for (ny, nz), offs in groups.items():
            m = ny * nz
            if len(offs) == 1:
                U = u[offs[0]:offs[0] + m].reshape(1, nz, ny, 3)
            else:
                idx = (torch.as_tensor(offs, device=u.device)[:, None] +
                       torch.arange(m, device=u.device)[None, :])
                U = u[idx.reshape(-1)].reshape(len(offs), nz, ny, 3)
            if ny % 2:
                U = torch.cat([U, U[:, :, -1:]], dim=2)
            if nz % 2:
                U = torch.cat([U, U[:, -1:]], dim=1)
            a, b = U[:, 0::2, 0::2], U[:, 0::2, 1::2]
            c, d = U[:, 1::2, 0::2], U[:, 1::2, 1::2]
            parts.append(torch.stack([nrm((b - a) + (d - c)), nrm((c - a) + (d - b)),
                                      nrm((a - b) + (d - c)),
                                      torch.maximum(nrm(d - a), nrm(c - b))]))
        row, col, mixed, diag = torch.stack(parts).amax(0).tolist()
        self._quad_steps = dict(row=row, col=col, mixed=mixed, diag=diag)
        return dict(self._quad_steps)


    def octets_fit(self):
        """True when every frame is whole 2x4 octets: rows of a multiple of 4
        pixels and an even number of rows."""
        return all(ny % 4 == 0 and nz % 2 == 0 for ny, nz in self.shapes)

    def octet_steps(self):
        """Departure from a plane of the FP64 unit vectors u to the pixels
        over the 2x4 octets of every frame (rows 2i, 2i+1, columns 4j..4j+3),
        as the octet kernels model them: the mean of the 8 u plus the mean
        row step times the column offset (-1.5..1.5) plus the mean column
        step times the row offset (-0.5, 0.5). Returns the largest norm of
        that residual (``plane``), the largest |u - mean| (``extent``) and
        the largest mean row / column step (``step``); None when a frame is
        not whole octets. Computed once per Pixels object."""
        if getattr(self, "_octet_steps", None) is not None:
            return dict(self._octet_steps)
        if not self.octets_fit():
            return None
        x = self.xyz
        u = x / torch.linalg.vector_norm(x, dim=1, keepdim=True)
        groups = {}
        for (off, m), shp in zip(self.spans, self.shapes):
            groups.setdefault(shp, []).append(off)
        parts = []
        mo = (torch.arange(4, device=u.device, dtype=u.dtype) - 1.5).view(1, 1, 1, 4, 1)
        to = (torch.arange(2, device=u.device, dtype=u.dtype) - 0.5).view(1, 2, 1, 1, 1)
        for (ny, nz), offs in groups.items():
            m = ny * nz
            if len(offs) == 1:
                U = u[offs[0]:offs[0] + m]
            else:
                idx = (torch.as_tensor(offs, device=u.device)[:, None] +
                       torch.arange(m, device=u.device)[None, :])
                U = u[idx.reshape(-1)]
            U = U.reshape(-1, 2, ny // 4, 4, 3)          # (row pairs, 2, octets, 4, 3)
            mean = U.mean(dim=(1, 3), keepdim=True)
            g = (U[:, :, :, 1:] - U[:, :, :, :-1]).mean(dim=(1, 3), keepdim=True)
            h = (U[:, 1:] - U[:, :1]).mean(dim=(1, 3), keepdim=True)
            res = U - (mean + mo * g + to * h)
            nrm = lambda t: torch.linalg.vector_norm(t, dim=-1).amax()
            parts.append(torch.stack([nrm(res), nrm(U - mean),
                                      torch.maximum(nrm(g), nrm(h))]))
        plane, extent, step = torch.stack(parts).amax(0).tolist()
        self._octet_steps = dict(plane=plane, extent=extent, step=step)
        return dict(self._octet_steps)

    def squares_fit(self):
        """True when every frame is whole 4x4 squares: a row length and a
        row count that are multiples of 4."""
        return all(ny % 4 == 0 and nz % 4 == 0 for ny, nz in self.shapes)

    def square_steps(self):
        """Departure from a plane of the FP64 unit vectors u to the pixels
        over the 4x4 squares of every frame (rows 4i..4i+3, columns
        4j..4j+3), exactly as the square kernels model them: the mean of the
        16 u plus the column offset (-1.5..1.5) times the mean row step of
        the four quads (their steps b - a and d - c) plus the row offset
        times their mean column step (c - a, d - b). Returns the largest
        norm of that residual (``plane``), the largest |u - mean|
        (``extent``) and the largest mean step (``step``); None when a frame
        is not whole squares. Computed once per Pixels object."""
        if getattr(self, "_square_steps", None) is not None:
            return dict(self._square_steps)
        if not self.squares_fit():
            return None
        x = self.xyz
        u = x / torch.linalg.vector_norm(x, dim=1, keepdim=True)
        groups = {}
        for (off, m), shp in zip(self.spans, self.shapes):
            groups.setdefault(shp, []).append(off)
        parts = []
        mo = (torch.arange(4, device=u.device, dtype=u.dtype) - 1.5).view(1, 1, 1, 4, 1)
        to = (torch.arange(4, device=u.device, dtype=u.dtype) - 1.5).view(1, 4, 1, 1, 1)
        nrm = lambda t: torch.linalg.vector_norm(t, dim=-1).amax()
        for (ny, nz), offs in groups.items():
            m = ny * nz
            if len(offs) == 1:
                U = u[offs[0]:offs[0] + m]
            else:
                idx = (torch.as_tensor(offs, device=u.device)[:, None] +
                       torch.arange(m, device=u.device)[None, :])
                U = u[idx.reshape(-1)]
            U = U.reshape(-1, 4, ny // 4, 4, 3)          # (row quads, 4, squares, 4, 3)
            mean = U.mean(dim=(1, 3), keepdim=True)
            # within-quad steps only: columns 0->1 and 2->3, rows 0->1 and 2->3
            g = (U[:, :, :, 1::2] - U[:, :, :, 0::2]).mean(dim=(1, 3), keepdim=True)
            h = (U[:, 1::2] - U[:, 0::2]).mean(dim=(1, 3), keepdim=True)
            res = U - (mean + mo * g + to * h)
            parts.append(torch.stack([nrm(res), nrm(U - mean),
                                      torch.maximum(nrm(g), nrm(h))]))
        plane, extent, step = torch.stack(parts).amax(0).tolist()
        self._square_steps = dict(plane=plane, extent=extent, step=step)
        return dict(self._square_steps)


@dataclass
class Atoms:
    """Atoms on the device in the frame of the pixels."""
    pos: torch.Tensor       # float64 (N, 3) [m]
    species: torch.Tensor   # int32 (N,)
    amp: torch.Tensor       # float32 (N, 2)
    counts: np.ndarray      # int64 (S,) atoms per species
    table: SpeciesTable
    extra: dict = field(default_factory=dict)

    @property
    def n(self):
        return int(self.pos.shape[0])


def atoms_lab(pos_A, species_idx, rot, trans, table, e0=None, grid=None, device="cuda",
              stream=None, counts=None):
    """Stage transform and incident amplitude on the device (mk_atoms_lab).

    ``pos_A`` (N,3) float32 Angstrom and ``species_idx`` (N,) may be host
    arrays or device tensors; with device species pass ``counts`` (atoms per
    species) so nothing is read back."""
    L = _require_cuda()
    pos_A = torch.as_tensor(pos_A)
    n = int(pos_A.shape[0])
    pin = pos_A.to(device=device, dtype=torch.float32).contiguous()
    pos = torch.empty((n, 3), dtype=torch.float64, device=device)
    amp = torch.empty((n, 2), dtype=torch.float32, device=device)
    rot = np.ascontiguousarray(rot, dtype=np.float32).reshape(9)
    trans = np.ascontiguousarray(trans, dtype=np.float32).reshape(3)
    e0_t, gny, gnz, g = None, 0, 0, None
    if e0 is not None:
        e0_t = torch.view_as_real(torch.as_tensor(np.ascontiguousarray(e0, dtype=np.complex64))).to(device)
        gny, gnz = int(e0.shape[0]), int(e0.shape[1])
        g = np.ascontiguousarray(grid, dtype=np.float64)
    check(L.mk_atoms_lab(n, _ptr(pin), rot.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                         trans.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), _ptr(e0_t), gny, gnz,
                         None if g is None else g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                         _ptr(pos), _ptr(amp), _stream_handle(stream)))
    if isinstance(species_idx, torch.Tensor):
        sp = species_idx.to(device=device, dtype=torch.int32).contiguous()
        if counts is None:
            counts = torch.bincount(sp.long(), minlength=len(table.labels)).cpu().numpy()
    else:
        sp = torch.as_tensor(np.ascontiguousarray(species_idx, dtype=np.int32)).to(device)
        if counts is None:
            counts = np.bincount(np.asarray(species_idx), minlength=len(table.labels))
    return Atoms(pos, sp, amp, np.asarray(counts, dtype=np.int64), table)


def depth_forward_factors(table):
    """(S, 2) float32 per species: f0(0) + f' and f'' (the forward factors of
    the transmission map, summed in float32 as Beam.py:7190-7197 does)."""
    re = table.f0z.astype(np.float32) + table.anom.real.astype(np.float32)
    return np.stack([re, table.anom.imag.astype(np.float32)], 1).astype(np.float32)


def _gauss_blur(m, rad):
    """Circular convolution with the reference's (2 rad + 1)^2 Gaussian placed
    at the map's corner (np.fft.fft2(k, s=shape), Beam.py:7268-7277)."""
    sig = rad / 2.0
    y, x = np.ogrid[-rad:rad + 1, -rad:rad + 1]
    k = np.exp(-(x * x + y * y) / (2.0 * sig * sig)).astype(np.float32)
    k /= k.sum()
    K = torch.zeros(m.shape, dtype=torch.float64, device=m.device)
    K[: 2 * rad + 1, : 2 * rad + 1] = torch.as_tensor(k.astype(np.float64))
    out = torch.fft.ifft2(torch.fft.fft2(m.double()) * torch.fft.fft2(K)).real
    return out.float().contiguous()


def depth_maps(atoms, grid_shape, grid, wavelength_A, kernel_radius=0, wrap=True, stream=None):
    """Attenuation and phase maps (tau, phi) of the whole sample on the beam
    grid, float32 device (NyB, NzB): column sums of the atoms' forward
    factors (mk_beam_column_sums), tau/phi (mk_beam_column_maps), the
    optional Gaussian blur of radius ``kernel_radius`` pixels, and with
    ``wrap`` the round trip through A = exp(-tau + i phi) the per-atom field
    reads (mk_beam_column_wrap)."""
    L = _require_cuda()
    ny, nz = int(grid_shape[0]), int(grid_shape[1])
    dev = atoms.pos.device
    f32 = dict(dtype=torch.float32, device=dev)
    sr, si = torch.empty((ny, nz), **f32), torch.empty((ny, nz), **f32)
    fwd = torch.as_tensor(depth_forward_factors(atoms.table)).to(dev)
    g = np.ascontiguousarray(grid, dtype=np.float64)
    gp = g.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    sh = _stream_handle(stream)
    check(L.mk_beam_column_sums(atoms.n, _ptr(atoms.pos), _ptr(atoms.species), _ptr(fwd),
                                int(fwd.shape[0]), ny, nz, gp, _ptr(sr), _ptr(si), sh))
    tau, phi = torch.empty((ny, nz), **f32), torch.empty((ny, nz), **f32)
    check(L.mk_beam_column_maps(ny, nz, _ptr(sr), _ptr(si), float(wavelength_A), float(g[0]),
                                float(g[1]), _ptr(tau), _ptr(phi), sh))
    if int(kernel_radius) > 0:
        rad = int(kernel_radius)
        if 2 * rad + 1 > min(ny, nz):
            raise ValueError(f"blur radius {rad} does not fit the {ny} x {nz} beam grid")
        phi = _gauss_blur(phi, rad)
        tau = torch.clamp_min(_gauss_blur(tau, rad), 0.0).contiguous()
    if wrap:
        check(L.mk_beam_column_wrap(ny, nz, _ptr(tau), _ptr(phi), sh))
    return tau, phi


def depth_bounds(atoms):
    """Front and back of the sample along the +x beam [A] as the float32 lab
    x the stage transform produced (Beam.py:5583-5618); (0, 1) when flat."""
    if atoms.n == 0:
        return 0.0, 1.0
    x = atoms.pos[:, 0]
    lo = float(np.float32(float(x.min()) * 1e10))
    hi = float(np.float32(float(x.max()) * 1e10))
    return (lo, hi) if hi > lo else (0.0, 1.0)


def ein_depth(atoms, e0, grid, tau, phi, s_min, s_max, stream=None):
    """Overwrite the atoms' amplitudes with the depth-dependent incident field
    (mk_atoms_ein_depth)."""
    L = _require_cuda()
    e0_t = torch.view_as_real(torch.as_tensor(np.ascontiguousarray(e0, dtype=np.complex64))).to(
        atoms.pos.device)
    g = np.ascontiguousarray(grid, dtype=np.float64)
    check(L.mk_atoms_ein_depth(atoms.n, _ptr(atoms.pos), _ptr(e0_t), _ptr(tau), _ptr(phi),
                               int(tau.shape[0]), int(tau.shape[1]),
                               g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), float(s_min),
                               float(s_max), _ptr(atoms.amp), _stream_handle(stream)))
    return atoms


class Tiles:
    """Species-partitioned, Morton-ordered atom tiles (mk_tiles_build)."""

    def __init__(self, atoms: Atoms, k, tile_atoms=DEFAULT_TILE_ATOMS, device="cuda", stream=None):
        L = _require_cuda()
        T = int(tile_atoms)
        counts = np.ascontiguousarray(atoms.counts, dtype=np.int64)
        n_tiles = int(sum((int(c) + T - 1) // T for c in counts))
        self.n_tiles, self.tile_atoms = n_tiles, T
        self.origin = torch.empty((max(n_tiles, 1), 4), dtype=torch.float64, device=device)
        self.species = torch.empty(max(n_tiles, 1), dtype=torch.int32, device=device)
        self.pos = torch.empty((max(n_tiles, 1) * T, 4), dtype=torch.float32, device=device)
        self.amp = torch.empty((max(n_tiles, 1) * T, 2), dtype=torch.float32, device=device)
        self.abi = MkTiles(n_tiles, T, self.origin.data_ptr(), self.species.data_ptr(),
                           self.pos.data_ptr(), self.amp.data_ptr())
        self.table = atoms.table
        if atoms.n == 0:
            return
        ws_n = L.mk_tiles_workspace_size(atoms.n)
        ws = torch.empty(ws_n, dtype=torch.uint8, device=device)
        check(L.mk_tiles_build(atoms.n, _ptr(atoms.pos), _ptr(atoms.species), _ptr(atoms.amp),
                               len(counts), counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                               float(k), ctypes.byref(self.abi), _ptr(ws), ws_n,
                               _stream_handle(stream)))
        self._ws = ws   # keep until the stream has consumed it

    def _extents(self):
        """(largest tile radius, largest origin norm), from the origins read
        back once per object (its arrays do not change after the build)."""
        if getattr(self, "_ext", None) is None:
            if not self.n_tiles:
                self._ext = (0.0, 0.0)
            else:
                o = origins_host(self)
                self._ext = (float(o[:, 3].max()), float(np.linalg.norm(o[:, :3], axis=1).max()))
        return self._ext

    def max_radius(self):
        return self._extents()[0]

    def max_origin_norm(self):
        return self._extents()[1]

    def amp_is_real(self):
        # atom pairs interleaved as re0 re1 im0 im1; one read-back per object
        if getattr(self, "_real", None) is None:
            self._real = bool((self.amp.view(-1, 4)[:, 2:] == 0).all()) if self.n_tiles else True
        return self._real


DEFAULT_LAUNCH = dict(pix_per_thread=4, threads=128, slices=0, pairs=0)


SQUARE_MAX_TILE_ATOMS = 1024


def default_launch(level=0, tile_atoms=None):
    """Untuned launch shape for a pixel-sharing level (0 none, 1 pairs, 2
    quads, 3 octets, 4 squares): quads run two per thread (8 pixels;
    measured 1.6-2 % above one on the 8.19M-atom exposure and the 128^2 scan
    frames), octets are 8 pixels a thread, squares 16. Squares only with
    tiles of at most SQUARE_MAX_TILE_ATOMS atoms (``tile_atoms``; None
    counts as DEFAULT_TILE_ATOMS): with larger tiles three 128-thread square
    blocks do not fit an SM's shared memory, and at two blocks the square
    kernel ran the 8.19M-atom exposure 1.5 % slower than octets, against
    12 % faster at three."""
    level = int(level)
    if level >= 4 and (tile_atoms or DEFAULT_TILE_ATOMS) > SQUARE_MAX_TILE_ATOMS:
        level = 3
    ppt = 16 if level >= 4 else 8 if level >= 2 else 4
    return dict(DEFAULT_LAUNCH, pairs=level, pix_per_thread=ppt)
FACTOR_TABLE_EXCURSION = 1e-6


def factor_table_ok(tiles, pix, phys):
    """Whether the split kernel may take each species' factor at the pixel's
    own direction (``Pixels.factor_table``) instead of at the direction to
    each tile: the two directions differ by at most 2 (|o| + r) / R0 (tile
    origin o, radius r, pixel distance R0), which must stay below
    FACTOR_TABLE_EXCURSION -- the bound the split form already keeps for the
    factor's change across a tile, 2 r / R0, with the tile origins added.
    Not with remove_forward, whose Q < Q_cut test stays per tile and pixel."""
    if phys.remove_forward or not tiles.n_tiles:
        return False
    r0 = max(pix.r0_min(), 1e-300)
    return 2.0 * (tiles.max_origin_norm() + tiles.max_radius()) / r0 < FACTOR_TABLE_EXCURSION


PAIR_DELTA_MAX = 0.5     # rad: the long pair polynomials are then exact to ~2e-6 per term
PAIR_SHORT_DELTA = 0.07  # rad: the short ones to 1e-6 (the kernel's MK_PAIR_SHORT_DELTA)


def _pair_rate(tiles, pix: Pixels, k):
    """Half phase difference of a pixel pair per metre of tile radius [rad/m]:
    (k/2) |u_a - u_b|, widened for the tile-origin term of w."""
    grow = 1.0 + 2.0 * tiles.max_origin_norm() / max(pix.r0_min(), 1e-300)
    return 0.5 * float(k) * pix.pair_step() * grow * 1.05


def pair_delta(tiles, pix: Pixels, k):
    """Bound on the half phase difference pi |D| |w_a - w_b| of a pixel pair
    over all tiles [rad]."""
    if not tiles.n_tiles:
        return 0.0
    return _pair_rate(tiles, pix, k) * tiles.max_radius()


def pair_short_radius(tiles, pix: Pixels, k):
    """Largest tile radius [m] whose pairs stay within PAIR_SHORT_DELTA."""
    if not tiles.n_tiles:
        return 0.0
    rate = _pair_rate(tiles, pix, k)
    return PAIR_SHORT_DELTA / rate if rate > 0 else 1.0


def pairs_allowed(tiles, pix: Pixels, k):
    return pair_delta(tiles, pix, k) <= PAIR_DELTA_MAX


def quad_bounds(tiles, pix: Pixels, k, fresnel_rad=0.0):
    """Error bounds of the 2x2 pixel-quad form over all tiles.

    ``delta`` [rad] bounds the two half differences u, v that go to the
    polynomials (as ``pair_delta`` does for pairs); ``short_radius_m`` is the
    largest tile radius whose u, v stay within PAIR_SHORT_DELTA; ``cross``
    [rad] bounds the phase the quad form drops: the mixed second difference
    (pi/2) D.(w_a + w_d - w_b - w_c), of order k |D| (pixel/distance)^2,
    widened for the tile-origin term of w, plus the change of the |d|^2 term
    across the quad, which the quad shares (2 ``fresnel_rad`` x the quad's
    diagonal step)."""
    st = pix.quad_steps()
    if not tiles.n_tiles:
        return dict(delta=0.0, short_radius_m=1.0, cross=0.0, **st)
    r0 = max(pix.r0_min(), 1e-300)
    o_ratio = tiles.max_origin_norm() / r0
    grow = 1.0 + 2.0 * o_ratio
    rate = 0.25 * float(k) * max(st["row"], st["col"]) * grow * 1.05
    r = tiles.max_radius()
    step = 0.5 * max(st["row"], st["col"])
    mixed = st["mixed"] * grow + 4.0 * o_ratio * step * step
    cross = 0.25 * float(k) * r * mixed * 1.05 + 2.0 * float(fresnel_rad) * st["diag"]
    return dict(delta=rate * r, short_radius_m=(PAIR_SHORT_DELTA / rate if rate > 0 else 1.0),
                cross=cross, **st)


OCTET_MIN_TILE_FRACTION = 0.5   # octets only where at least half the tiles take them


def octet_bounds(tiles, pix: Pixels, k, budget_rad, fresnel_rad=0.0):
    """Largest tile radius [m] whose 2x4 pixel-octet form stays within the
    phase budget, or None when a frame is not whole octets.

    The octet drops, beyond the quad form, the departure of w over its 8
    pixels from a plane (mean, mean row step, mean column step): the kernel
    takes both quads' half differences from the octet's mean steps and their
    phases from the octet's mean phase. That residual of the FP64 pixel
    directions (``Pixels.octet_steps``), widened for the tile-origin term of
    w, times k |D| <= k r bounds the phase error of a tile of radius r; the
    |d|^2 term, which the octet evaluates once at its centre, adds
    4 ``fresnel_rad`` x the octet's extent |u - mean|. Tiles wider than the
    returned radius take the quad form inside the octet kernel. Returns
    dict(radius_m, cross (the bound at min(radius, widest tile)), plane,
    extent, step)."""
    st = pix.octet_steps()
    if st is None:
        return None
    r0 = max(pix.r0_min(), 1e-300)
    o_ratio = tiles.max_origin_norm() / r0 if tiles.n_tiles else 0.0
    grow = 1.0 + 2.0 * o_ratio
    plane = st["plane"] * grow + 12.0 * o_ratio * st["step"] ** 2
    rate = float(k) * plane * 1.05                      # rad per metre of tile radius
    fixed = 4.0 * float(fresnel_rad) * st["extent"]
    room = float(budget_rad) - fixed
    radius = room / rate if (room > 0.0 and rate > 0.0) else (1.0 if room > 0.0 else 0.0)
    r_eff = min(radius, tiles.max_radius()) if tiles.n_tiles else 0.0
    return dict(radius_m=radius, cross=rate * r_eff + fixed, **st)


def square_bounds(tiles, pix: Pixels, k, budget_rad, fresnel_rad=0.0):
    """Largest tile radius [m] whose 4x4 pixel-square form stays within the
    phase budget, or None when a frame is not whole squares.

    As ``octet_bounds`` for the square's 16 pixels: the residual of the FP64
    pixel directions from the kernel's plane (``Pixels.square_steps``),
    widened for the tile-origin term of w -- whose part quadratic in the
    pixel offsets (m, t) (columns and rows, -1.5..1.5 steps s) is
    (m^2 (g.o) g + t^2 (h.o) h + m t ((g.o) h + (h.o) g)) / |P|, off the
    plane by at most (1 + 1 + 2 x 2.25) |o| s^2 / |P| over the square (2.5
    over an octet, where the bound takes 12: the same margin gives 32) --
    times k r, plus 4 ``fresnel_rad`` x the square's extent for the |d|^2
    term taken at its centre. Tiles wider than the returned radius take the
    quad form inside the square kernel. Returns dict(radius_m, cross (the
    bound at min(radius, widest tile)), plane, extent, step)."""
    st = pix.square_steps()
    if st is None:
        return None
    r0 = max(pix.r0_min(), 1e-300)
    o_ratio = tiles.max_origin_norm() / r0 if tiles.n_tiles else 0.0
    grow = 1.0 + 2.0 * o_ratio
    plane = st["plane"] * grow + 32.0 * o_ratio * st["step"] ** 2
    rate = float(k) * plane * 1.05                      # rad per metre of tile radius
    fixed = 4.0 * float(fresnel_rad) * st["extent"]
    room = float(budget_rad) - fixed
    radius = room / rate if (room > 0.0 and rate > 0.0) else (1.0 if room > 0.0 else 0.0)
    r_eff = min(radius, tiles.max_radius()) if tiles.n_tiles else 0.0
    return dict(radius_m=radius, cross=rate * r_eff + fixed, **st)


def origins_host(tiles):
    """(n_tiles, 4) float64 tile origins and radii on the host: one
    read-back per tiles object, which the extents and the fractions of tiles
    within the pixel-sharing radii all use."""
    h = getattr(tiles, "_origins_host", None)
    if h is None:
        h = (tiles.origin[: tiles.n_tiles].cpu().numpy() if tiles.n_tiles
             else np.zeros((0, 4), dtype=np.float64))
        tiles._origins_host = h
    return h


def tile_fraction_within(tiles, radius_m):
    """Fraction of the tiles whose radius is at most ``radius_m``."""
    if not tiles.n_tiles:
        return 1.0
    return float((origins_host(tiles)[:, 3] <= float(radius_m)).mean())


def pixel_grouping(tiles, pix: Pixels, k, budget_rad, fresnel_rad=0.0, analyser=False):
    """Widest legal sharing of one sin/cos between neighbouring pixels:
    (level, info) with level 4 squares, 3 octets, 2 quads, 1 pairs, 0 none, and
    info["pairs_ok"] whether pairs alone are legal. Pairs need ``pair_delta``
    <= PAIR_DELTA_MAX (a pair across a row end, with an odd row length,
    breaks it); quads need their half differences within it and their
    dropped phase within ``budget_rad``, on any detector shape; octets (2x4:
    two quads sharing their half differences) need frames of whole octets
    and at least OCTET_MIN_TILE_FRACTION of the tiles narrow enough for
    their dropped phase to fit the budget (``octet_bounds``; the wider tiles
    take the quad form); squares (4x4: four quads sharing them) need that
    and the same of frames of whole squares and of their own radius
    (``square_bounds``). ``analyser`` (0 off,
    1 top-hat, 2 Darwin): the analyser kernels have quads for the top-hat
    (tiles the acceptance edge cuts take the per-atom loop) and no pairs or
    octets; a Darwin analyser expands per atom on every tile, so it shares
    nothing."""
    analyser = int(analyser)
    info = dict(pair_delta_rad=pair_delta(tiles, pix, k))
    info["pairs_ok"] = (not analyser) and info["pair_delta_rad"] <= PAIR_DELTA_MAX
    if analyser == 2:
        return 0, info
    q = quad_bounds(tiles, pix, k, fresnel_rad)
    info.update(quad_delta_rad=q["delta"], quad_cross_rad=q["cross"],
                quad_short_radius_m=q["short_radius_m"])
    if q["delta"] <= PAIR_DELTA_MAX and q["cross"] <= budget_rad:
        if not analyser:
            ob = octet_bounds(tiles, pix, k, budget_rad, fresnel_rad)
            if ob is not None and ob["radius_m"] > 0.0:
                frac = tile_fraction_within(tiles, ob["radius_m"])
                info.update(octet_cross_rad=ob["cross"], octet_radius_m=ob["radius_m"],
                            octet_tile_fraction=frac)
                if frac >= OCTET_MIN_TILE_FRACTION:
                    sb = square_bounds(tiles, pix, k, budget_rad, fresnel_rad)
                    if sb is not None and sb["radius_m"] > 0.0:
                        sfrac = tile_fraction_within(tiles, sb["radius_m"])
                        info.update(square_cross_rad=sb["cross"], square_radius_m=sb["radius_m"],
                                    square_tile_fraction=sfrac)
                        if sfrac >= OCTET_MIN_TILE_FRACTION:
                            return 4, info
                    return 3, info
        return 2, info
    return (1 if info["pairs_ok"] else 0), info


def analyser_launch(cfg):
    """A launch shape the analyser kernels have: quads with 128/256 threads
    and 4/8 pixels, else one sin/cos per term with ANALYSER_LAUNCHES."""
    cfg = dict(cfg)
    nt, ppt = int(cfg.get("threads", 128)), int(cfg.get("pix_per_thread", 4))
    if int(cfg.get("pairs", 0) or 0) in (3, 4):
        cfg["pairs"] = 2
    if int(cfg.get("pairs", 0) or 0) == 2:
        if nt not in (128, 256) or ppt not in (4, 8):
            cfg.update(threads=128, pix_per_thread=8)
    elif (nt, ppt) not in ANALYSER_LAUNCHES:
        cfg.update(threads=128, pix_per_thread=4)
    return cfg


def grouping_launch(cfg, level, tiles, pix, k, info):
    """Clamp a launch dict's ``pairs`` to the legal ``level`` and the pixels
    per thread the kernels have (quads: 4 or 8; pairs: even, and only where
    ``info["pairs_ok"]``), and set the short-polynomial radius for the mode
    kept."""
    cfg = dict(cfg)
    pairs_ok = bool(info.get("pairs_ok", level >= 1))
    mode = min(int(cfg.get("pairs", 0) or 0), int(level))
    ppt = int(cfg.get("pix_per_thread", 4))
    if mode == 4 and (ppt != 16 or int(cfg.get("threads", 128)) not in (128, 192)):
        mode = 3
    if mode < 4 and (ppt == 16 or int(cfg.get("threads", 128)) == 192):
        # 16 pixels a thread and 192-thread blocks exist only as squares
        ppt = 8 if mode >= 2 else 4
        cfg["pix_per_thread"] = ppt
        if int(cfg.get("threads", 128)) == 192:
            cfg["threads"] = 128
    if mode == 3 and ppt != 8:
        mode = 2
    if mode == 2 and ppt not in (4, 8):
        mode = 1
    if mode == 1 and (ppt % 2 or not pairs_ok):
        mode = 0
    cfg["pairs"] = mode
    cfg["octet_radius_m"] = (float(info.get("octet_radius_m", 0.0)) if mode == 3 else
                             float(info.get("square_radius_m", 0.0)) if mode == 4 else 0.0)
    if mode >= 2:
        cfg["pair_short_radius_m"] = info["quad_short_radius_m"]
    elif mode == 1:
        cfg["pair_short_radius_m"] = pair_short_radius(tiles, pix, k)
    else:
        cfg["pair_short_radius_m"] = 0.0
    return cfg


def run_split(tiles: Tiles, pix: Pixels, phys, table: SpeciesTable, launch=None, fresnel=-1,
              amp_real=None, out=None, accumulate=False, stream=None, fresnel_radius=0.0,
              factor_table=None):
    """FP32 split-phase sum; returns float64 (P, 2) (a view of `out` if given).
    ``factor_table`` None: the per-(species, pixel) factor table where
    ``factor_table_ok`` admits it (else the factor per tile and pixel);
    False: never; True: always.
    With ``fresnel`` set, only tiles wider than ``fresnel_radius`` [m] keep the
    |d|^2 term (0: all tiles). ``launch["pairs"]`` = 1 shares one sin/cos
    between pixels 2j and 2j+1; only legal where ``pairs_allowed`` holds;
    ``launch["pair_short_radius_m"]`` (``pair_short_radius``) then selects
    the short delta polynomial for the tiles up to that radius."""
    L = _require_cuda()
    cfg = dict(DEFAULT_LAUNCH, **(launch or {}))
    pairs = int(cfg.get("pairs", 0) or 0)
    short_r = 0.0
    if pairs:
        short_r = cfg.get("pair_short_radius_m")
        if short_r is None:
            short_r = (quad_bounds(tiles, pix, phys.k)["short_radius_m"] if pairs >= 2
                       else pair_short_radius(tiles, pix, phys.k))
    ln = MkLaunch(int(cfg["pix_per_thread"]), int(cfg["threads"]), int(cfg["slices"]), int(fresnel),
                  int(tiles.amp_is_real() if amp_real is None else bool(amp_real)),
                  float(fresnel_radius), int(pairs), short_r,
                  float(cfg.get("sin_direct_max_rad", 0.0) or 0.0),
                  float(cfg.get("octet_radius_m", 0.0) or 0.0))
    wsb = ctypes.c_size_t(0)
    check(L.mk_split_plan(ctypes.byref(tiles.abi), ctypes.byref(pix.abi), ctypes.byref(ln),
                          ctypes.byref(wsb)))
    ws_n = int(wsb.value)
    ws = torch.empty(ws_n, dtype=torch.uint8, device=pix.xyz.device)
    if out is None:
        out = torch.zeros((pix.n, 2), dtype=torch.float64, device=pix.xyz.device)
    sp = table.abi()
    use_tab = factor_table_ok(tiles, pix, phys) if factor_table is None else bool(factor_table)
    pabi, ftab = pix.abi, None
    if use_tab:
        ftab = pix.factor_table(table, phys, stream)
        pabi = MkPixels.from_buffer_copy(pix.abi)
        pabi.factor = ftab.data_ptr()
    check(L.mk_kin_split_f32(ctypes.byref(tiles.abi), ctypes.byref(sp), ctypes.byref(phys),
                             ctypes.byref(pabi), ctypes.byref(ln), _ptr(out), int(bool(accumulate)),
                             _ptr(ws), ws_n, _stream_handle(stream)))
    out._mk_keep = (ws, ftab)
    return out


def run_plain(atoms: Atoms, pix: Pixels, phys, slices=0, out=None, accumulate=False, stream=None):
    """FP64 plain sum; returns float64 (P, 2)."""
    L = _require_cuda()
    n = atoms.n
    if slices > 0:
        ns = int(slices)
    else:
        sms = torch.cuda.get_device_properties(pix.xyz.device).multi_processor_count
        bx = (pix.n + 127) // 128
        ns = max(1, min((8 * sms + bx - 1) // bx, (n + 511) // 512, 4096))
    ws_n = L.mk_sum_workspace_size(pix.n, ns)
    ws = torch.empty(ws_n, dtype=torch.uint8, device=pix.xyz.device)
    if out is None:
        out = torch.zeros((pix.n, 2), dtype=torch.float64, device=pix.xyz.device)
    sp = atoms.table.abi()
    check(L.mk_kin_plain_f64(n, _ptr(atoms.pos), _ptr(atoms.species), _ptr(atoms.amp),
                             ctypes.byref(sp), ctypes.byref(phys), ctypes.byref(pix.abi), ns,
                             _ptr(out), int(bool(accumulate)), _ptr(ws), ws_n,
                             _stream_handle(stream)))
    out._mk_keep = ws
    return out


def sync(stream=None):
    """Wait for the stream and raise on a device-side error flag."""
    L = _require_cuda()
    check(L.mk_sync_status(_stream_handle(stream)))


class TilesView:
    """The first ``m`` tiles of a Tiles object (same device buffers)."""

    def __init__(self, tiles, m):
        self.n_tiles, self.tile_atoms = int(m), tiles.tile_atoms
        self.origin, self.species, self.pos, self.amp = tiles.origin, tiles.species, tiles.pos, tiles.amp
        self.table = tiles.table
        self.abi = MkTiles(self.n_tiles, self.tile_atoms, self.origin.data_ptr(),
                           self.species.data_ptr(), self.pos.data_ptr(), self.amp.data_ptr())

    def amp_is_real(self):
        if getattr(self, "_real", None) is None:
            self._real = bool((self.amp[: self.n_tiles * self.tile_atoms].reshape(-1, 4)[:, 2:]
                               == 0).all())
        return self._real

    def _extents(self):
        """(largest tile radius, largest origin norm), from the origins read
        back once per object (its arrays do not change after the build)."""
        if getattr(self, "_ext", None) is None:
            if not self.n_tiles:
                self._ext = (0.0, 0.0)
            else:
                o = origins_host(self)
                self._ext = (float(o[:, 3].max()), float(np.linalg.norm(o[:, :3], axis=1).max()))
        return self._ext

    def max_radius(self):
        return self._extents()[0]

    def max_origin_norm(self):
        return self._extents()[1]
