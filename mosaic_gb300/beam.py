"""``beam``: the drop-in for the reference's kinematic scattering entry point.

Mirrors the public surface of MOSAIC's ``beam`` class that the kinematic path
uses (Beam.py:59-310, 1047-1156, 6028-6496, 7771-7824): ``create_beam``,
``set_wavefield``, ``set_phase_tolerance``, ``atomic_scattering_kinematic``,
``interact_beam_gpu``, ``atomic_direct_interaction`` -- same arguments, same
(Nz, Ny) complex64 result, same sample/detector/stage duck types and the same
error behaviour (ValueError for a non-+x beam or size mismatches,
MemoryError when scratch cannot be allocated).

Arithmetic runs on the GPU in libmosaic_kin.so:
  * ``_use_fast_kernel`` True (default): FP32 split-phase sum
    (``mk_kin_split_f32``); it declines to the FP64 sum when the geometry
    leaves its error budget (extreme near field), as the reference's fast
    kernel declines to its general kernel (Beam.py:1376-1441).
  * ``_use_fast_kernel`` False: FP64 plain sum (``mk_kin_plain_f64``), the
    reference CPU kernel's arithmetic term for term.
There is no CPU path: ``use_gpu=False`` and a missing GPU raise.
"""
from __future__ import annotations

import hashlib
import os
import types
import warnings

import numpy as np
import torch

from . import engine
from .geometry import polarization_from_rate, polarization_state
from .tables import ScatteringTables, anomalous_at, f0_at_zero


class beam:
    """X-ray beam along +x and the kinematic scattering it produces."""

    def __init__(self, directory=None, tables: ScatteringTables | None = None):
        self.directory = directory
        self._direction = None
        self._energy = None
        self._wavelength = None
        self._pol_perp_rate = 0.5
        self._pol_direction = None
        self._pol_degree = None
        self._h = 6.62607015e-34
        self._c = 299792458
        self._q = 1.602176634e-19
        self._hq = self._h / self._q
        self._phase_tol_rad = 1e-3
        # FP32 path: phase budget for every dropped term of the split phase
        # (the reference's _kernel_phase_tol_rad, Beam.py:1404-1406).
        self._use_fast_kernel = True
        self._kernel_phase_tol_rad = 1e-6
        self._kernel_tile_atoms = None      # None: autotuned (512 untuned)
        self._kernel_launch = None          # None: autotuned
        # tune tile size and launch shape on the first use of a detector size
        # (as the reference tunes its fast kernel on first use, Beam.py:8871-8940);
        # MOSAIC_GB300_AUTOTUNE=0 uses the cached choice or the defaults only
        self._autotune = os.environ.get("MOSAIC_GB300_AUTOTUNE", "1") != "0"
        self.last_tune = []
        self._debye_waller = None           # element -> B [A^2]; None = no factor
        self.tables = tables or ScatteringTables()
        self.last_run = {}
        self._pix_cache = None

    # ------------------------------------------------------------ beam setup
    def create_beam(self, energy, eV=True, beam_shape="rectangular", beam_size=(1000.0, 1000.0),
                    beam_samples=(256, 256), beam_profile="uniform", gaussian_waist=None,
                    pol_perp_rate=0.5, pol_direction=None, pol_degree=None):
        """+x beam of the given energy and its transverse grid (Beam.py:151-218)."""
        self._direction = np.array([1.0, 0.0, 0.0], dtype=np.float32)
        if not eV:
            energy = energy / self._q
        self._energy = float(energy)
        self._wavelength = self._hq * self._c / self._energy
        k = 2.0 * np.pi / self._wavelength
        self._kx_scalar = np.float32(k)
        self._ky_scalar = np.float32(0.0)
        self._kz_scalar = np.float32(0.0)
        self._beam_shape = str(beam_shape).lower()
        self._beam_size = (float(beam_size[0]), float(beam_size[1]))
        self._beam_samples = (int(beam_samples[0]), int(beam_samples[1]))
        self._beam_profile = str(beam_profile).lower()
        self._gauss_waist = gaussian_waist
        self._set_polarization(pol_perp_rate, pol_direction, pol_degree)
        self._beam_e1 = np.array([0.0, 1.0, 0.0], dtype=np.float32)
        self._beam_e2 = np.array([0.0, 0.0, 1.0], dtype=np.float32)
        self._init_beam_grid()

    def _init_beam_grid(self):
        """Centred (u, v) grid and the zero-phase field map (Beam.py:220-264)."""
        Ny, Nz = self._beam_samples
        Sy, Sz = self._beam_size
        Ny, Nz = int(max(1, Ny)), int(max(1, Nz))
        self._beam_Ny, self._beam_Nz = Ny, Nz
        self._beam_du = float(Sy) / Ny
        self._beam_dv = float(Sz) / Nz
        self._beam_uc = (Ny - 1) * 0.5
        self._beam_vc = (Nz - 1) * 0.5
        u = (np.arange(Ny, dtype=np.float32) - self._beam_uc) * self._beam_du
        v = (np.arange(Nz, dtype=np.float32) - self._beam_vc) * self._beam_dv
        U, V = np.meshgrid(u, v, indexing="ij")
        if self._beam_shape == "circular":
            mask = ((U / max(0.5 * Sy, 1e-9)) ** 2 + (V / max(0.5 * Sz, 1e-9)) ** 2) <= 1.0
        else:
            mask = np.ones_like(U, dtype=bool)
        if self._beam_profile == "gaussian":
            wy, wz = self._gauss_waist if self._gauss_waist is not None else (0.5 * Sy, 0.5 * Sz)
            wy, wz = max(float(wy), 1e-6), max(float(wz), 1e-6)
            A0 = np.exp(-((U / wy) ** 2 + (V / wz) ** 2)).astype(np.float32)
            A0 *= mask.astype(np.float32)
        else:
            A0 = mask.astype(np.float32)
        self._beam_u_centers = u
        self._beam_v_centers = v
        self._beam_E0_map = (A0.astype(np.float32) + 0.0j).astype(np.complex64)

    def set_wavefield(self, wavefield):
        """User-supplied E0(u, v) on the beam grid (Beam.py:266-310)."""
        arr = np.asarray(wavefield)
        expected = (int(self._beam_Ny), int(self._beam_Nz))
        if arr.ndim != 2:
            raise ValueError(f"set_wavefield: expected a 2-D array of shape {expected}, got ndim={arr.ndim}")
        if tuple(arr.shape) != expected:
            raise ValueError(f"set_wavefield: expected shape {expected} (beam_samples), got {tuple(arr.shape)}")
        arr = np.ascontiguousarray(arr, dtype=np.complex64)
        if not (np.all(np.isfinite(arr.real)) and np.all(np.isfinite(arr.imag))):
            raise ValueError("set_wavefield: wavefield contains non-finite values (NaN/Inf)")
        self._beam_E0_map = arr
        self._beam_profile = "custom-" + hashlib.sha1(arr.tobytes()).hexdigest()[:12]

    def _set_polarization(self, pol_perp_rate, pol_direction=None, pol_degree=None):
        self._pol_perp_rate = float(np.clip(pol_perp_rate, 0.0, 1.0))
        self._pol_direction = (None if pol_direction is None
                               else np.asarray(pol_direction, dtype=np.float64).reshape(3))
        self._pol_degree = None if pol_degree is None else float(np.clip(pol_degree, 0.0, 1.0))

    def _polarization_state(self):
        """(p, ex, ey, ez) of the incident polarization (Beam.py:117-149)."""
        return polarization_state(self._pol_perp_rate, self._pol_direction, self._pol_degree,
                                  getattr(self, "_direction", None)
                                  if getattr(self, "_direction", None) is not None else (1, 0, 0))

    def set_phase_tolerance(self, phi_tol_rad: float):
        """Maximum phase error per contribution; invalid values mean 1e-3 rad."""
        try:
            val = float(phi_tol_rad)
            if not (val > 0.0):
                val = 1e-3
        except Exception:
            val = 1e-3
        self._phase_tol_rad = val

    def set_debye_waller(self, b_factors=None):
        """Per-element Debye-Waller B [A^2]: each scattering factor is multiplied
        by exp(-B s^2), s = sin(theta)/lambda. None (default) applies no factor,
        which is the reference's behaviour (thermal motion enters there only as
        explicit displacements)."""
        self._debye_waller = None if not b_factors else {str(k): float(v) for k, v in b_factors.items()}

    def _require_forward_beam(self, k_vec=None):
        """Refuse a beam that is not along +x (Beam.py:1132-1156)."""
        kx, ky, kz = ((self._kx_scalar, self._ky_scalar, self._kz_scalar) if k_vec is None else k_vec)
        kx, ky, kz = float(kx), float(ky), float(kz)
        if kx <= 0.0 or abs(ky) > 1e-6 * kx or abs(kz) > 1e-6 * kx:
            raise ValueError(
                "The scattering kernels assume a beam along +x (they take |k| from kx and the "
                f"incident phase as k*x); got k = ({kx:.4e}, {ky:.4e}, {kz:.4e}) 1/m.  Rotate the "
                "sample and detector with the stage instead of tilting the beam.")

    # ------------------------------------------------------- tables (parity)
    def parse_f0_db_all(self, database_name="f0_WaasKirf.dat"):
        return self.tables.f0

    def parse_f1f2_db_all(self, database_name="f1f2_CromerLiberman.dat"):
        return self.tables.f1f2

    @staticmethod
    def get_f1f2_from_params(energy, f1f2_table):
        return anomalous_at(energy, f1f2_table)

    @staticmethod
    def _build_f0_zero_dict(db_dict_f0_all):
        return {el: f0_at_zero(p) for el, p in db_dict_f0_all.items()}

    # --------------------------------------------------------------- staging
    @property
    def k(self):
        return 2.0 * np.pi / self._wavelength

    def _beam_grid(self):
        return (self._beam_du, self._beam_dv, self._beam_uc, self._beam_vc)

    def collect_atoms(self, sample):
        """Host arrays of every chunk: positions (N,3) float32 A and global
        species indices, labels without an f0 table dropped (they scatter
        nothing in the reference either, Beam.py:5679-5681)."""
        n_chunks = int(sample.chunk_total or 0)
        pos_list, idx_list, labels = [], [], []
        lab_index = {}
        for cid in range(1, n_chunks + 1):
            codes, lab, pos = self._load_chunk(sample, cid)
            if codes.size == 0:
                continue
            remap = np.full(len(lab), -1, dtype=np.int32)
            for i, el in enumerate(lab):
                if not self.tables.has(el):
                    continue
                if el not in lab_index:
                    lab_index[el] = len(labels)
                    labels.append(el)
                remap[i] = lab_index[el]
            g = remap[codes]
            keep = g >= 0
            if not keep.all():
                pos, g = pos[keep], g[keep]
            pos_list.append(pos)
            idx_list.append(g)
        if not pos_list:
            return np.zeros((0, 3), np.float32), np.zeros(0, np.int32), labels
        return np.concatenate(pos_list), np.concatenate(idx_list), labels

    def _load_chunk(self, sample, cid):
        """(codes, labels, positions float32) of one chunk, host side."""
        try:
            codes, lab = sample.load_chunk_species(cid, use_gpu=False, codes=True)
            codes = np.asarray(codes)
            lab = np.asarray(lab).astype(str)
        except TypeError:
            spc = np.asarray(sample.load_chunk_species(cid, use_gpu=False)).astype(str)
            lab, codes = np.unique(spc, return_inverse=True)
            codes = codes.reshape(-1)
        pos = np.zeros((0, 3), np.float32)
        if codes.size:
            try:      # this library's samples hand out their arrays without a copy
                pos = sample.load_chunk_positions(cid, use_gpu=False, copy=False)
            except TypeError:
                pos = sample.load_chunk_positions(cid, use_gpu=False)
            pos = np.asarray(pos, dtype=np.float32)
        if pos.shape[0] != codes.shape[0]:
            raise ValueError(f"positions/species size mismatch for chunk {cid}")
        return codes, lab, pos

    def stream_atoms(self, sample, device="cuda"):
        """Chunks straight into device arrays, without a host-side copy of the
        whole sample: one worker thread reads chunk i+1 (file read, thermal
        draw) while chunk i goes host -> device. The copies read the chunk's
        own (pageable) host arrays: on a Grace-Blackwell node the copy engines
        read pageable memory over NVLink-C2C at ~175 GB/s (measured on a
        GB300: 98 MB in 0.56 ms, against 0.48 ms from pinned memory), so the
        host copy into pinned staging buffers that a PCIe host needs would
        only add time. Returns device positions (N, 3) float32 A, species
        indices (N,) int32, the labels and the atoms per label."""
        from concurrent.futures import ThreadPoolExecutor
        n_chunks = int(sample.chunk_total or 0)
        sizes = [int(sample.chunk_atom_count(c)) for c in range(1, n_chunks + 1)]
        n_max = sum(sizes)
        dev = torch.device(device)
        pos_d = torch.empty((max(n_max, 1), 3), dtype=torch.float32, device=dev)
        idx_d = torch.empty(max(n_max, 1), dtype=torch.int32, device=dev)
        labels, lab_index = [], {}
        off = 0
        self.last_stream_bytes = 0               # host -> device bytes of this call
        # one loader thread, kept by the beam for later calls (a one-chunk
        # sample is read in place: there is nothing to overlap it with)
        ex = getattr(self, "_loader", None)
        if ex is None and n_chunks > 1:
            ex = self._loader = ThreadPoolExecutor(max_workers=1)
        submit = (ex.submit if n_chunks > 1 else
                  lambda fn, *a: types.SimpleNamespace(result=lambda r=fn(*a): r))
        nxt = submit(self._load_chunk, sample, 1) if n_chunks else None
        for cid in range(1, n_chunks + 1):
            codes, lab, pos = nxt.result()
            nxt = submit(self._load_chunk, sample, cid + 1) if cid < n_chunks else None
            if codes.size == 0:
                continue
            remap = np.full(len(lab), -1, dtype=np.int32)
            for i, el in enumerate(lab):
                if not self.tables.has(el):
                    continue
                if el not in lab_index:
                    lab_index[el] = len(labels)
                    labels.append(el)
                remap[i] = lab_index[el]
            # byte codes of known labels go to the device as they are and
            # are mapped to the global species there; anything else is
            # mapped (and filtered) on the host
            on_device = codes.dtype == np.uint8 and bool((remap >= 0).all())
            g = None
            if not on_device:
                g = remap[codes]
                keep = g >= 0
                if not keep.all():
                    pos, g = pos[keep], g[keep]
            n = int(pos.shape[0])
            if n == 0:
                continue
            # synchronous copies from pageable memory: the host arrays may
            # be reused as soon as each returns
            pos_d[off:off + n].copy_(torch.from_numpy(np.ascontiguousarray(pos, dtype=np.float32)))
            self.last_stream_bytes += 12 * n + (n + 4 * len(remap) if on_device else 4 * n)
            if on_device:
                lut = torch.from_numpy(remap).to(dev)
                raw = torch.from_numpy(np.ascontiguousarray(codes)).to(dev)
                idx_d[off:off + n] = lut[raw.long()]
            else:
                idx_d[off:off + n].copy_(torch.from_numpy(np.ascontiguousarray(g, dtype=np.int32)))
            off += n
        counts = (torch.bincount(idx_d[:off].long(), minlength=len(labels)).cpu().numpy()
                  if off and labels else np.zeros(len(labels), dtype=np.int64))
        return pos_d[:off], idx_d[:off], labels, counts.astype(np.int64)

    def stage_atoms(self, sample, stage, device="cuda"):
        """All atoms on the device, lab frame, with their incident amplitudes
        (chunks streamed to the device by ``stream_atoms``)."""
        pos, idx, labels, counts = self.stream_atoms(sample, device)
        table = engine.SpeciesTable.build(labels or ["H"], self.tables, self._energy,
                                          self._debye_waller)
        if not labels:
            counts = np.zeros(1, dtype=np.int64)
        return engine.atoms_lab(pos, idx, stage.rotation, stage.translation, table,
                                e0=self._beam_E0_map, grid=self._beam_grid(), device=device,
                                counts=counts)

    def apply_depth_ein(self, atoms, kernel_radius=0):
        """Depth-dependent incident field (Beam.py:4963-5140): the transmission
        maps of the staged sample itself, its depth window, and the per-atom
        amplitudes E0 exp(-f tau) exp(i f phi), in place on ``atoms``.
        Returns (tau, phi, (s_min, s_max))."""
        self._require_forward_beam()
        tau, phi = engine.depth_maps(atoms, self._beam_E0_map.shape, self._beam_grid(),
                                     self._wavelength * 1e10, kernel_radius)
        s_min, s_max = engine.depth_bounds(atoms)
        engine.ein_depth(atoms, self._beam_E0_map, self._beam_grid(), tau, phi, s_min, s_max)
        return tau, phi, (s_min, s_max)

    def depth_ein_maps(self, sample, stage, kernel_radius=0):
        """The transmission map A(u, v) = exp(-tau + i phi) (complex64 host,
        _compute_beam_column_A_map_*, Beam.py:7118-7283) and the depth window
        (_compute_global_depth_bounds, Beam.py:5583-5618) of a sample."""
        atoms = self.stage_atoms(sample, stage)
        tau, phi = engine.depth_maps(atoms, self._beam_E0_map.shape, self._beam_grid(),
                                     self._wavelength * 1e10, kernel_radius, wrap=False)
        A = torch.polar(torch.exp(-tau.double()), phi.double()).to(torch.complex64)
        return A.cpu().numpy(), engine.depth_bounds(atoms)

    def physics(self, apply_polarization=False, spherical_decay=False, remove_forward=False,
                beam_dir=(1.0, 0.0, 0.0), pol=None, analyser=None):
        return engine.physics(self.k, beam_dir, apply_polarization,
                              self._polarization_state() if pol is None else pol,
                              spherical_decay, remove_forward, analyser)

    @staticmethod
    def analyser_budget(tiles, r0_min, phys):
        """Largest relative error of the Darwin factor's first-order expansion
        across a tile (the split kernel's per-atom form):
        0.6 (rho / (R0 hw))^2 for tiles of radius rho; 0 otherwise (top-hat
        tiles are classified exactly)."""
        if phys.analyser == 2 and phys.analyser_halfwidth > 0.0:
            rho = tiles.max_radius()
            return 0.6 * (rho / (max(r0_min, 1e-30) * phys.analyser_halfwidth)) ** 2
        return 0.0

    # ---------------------------------------------------------- the sum
    def split_budget(self, tiles, r0_min):
        """Largest phase error [rad] of the terms the FP32 split form drops,
        and whether the |d|^2 (Fresnel) term must be kept.

        Dropped always: the third-order remainders k r^3 / R0^2 of the tile
        and origin expansions and the factor change across a tile. Dropped
        when ``fresnel`` is False: k r^2 / 2 R0.
        """
        k = self.k
        r = tiles.max_radius()
        o = tiles.max_origin_norm()
        r0 = max(r0_min, 1e-30)
        third = k * (r ** 3 + o ** 3 + 3 * o * o * r) / r0 ** 2
        fresnel_term = k * r * r / (2.0 * r0)
        tol = min(float(self._kernel_phase_tol_rad), float(self._phase_tol_rad))
        # tiles of radius above this keep the |d|^2 term, the rest drop it
        fresnel_radius = float(np.sqrt(2.0 * r0 * tol / k))
        return third, fresnel_term > tol, tol, dict(tile_radius_m=r, origin_max_m=o,
                                                    third_order_rad=third,
                                                    fresnel_rad=fresnel_term,
                                                    fresnel_radius_m=fresnel_radius)

    MAX_SPLIT_DEPTH = 6

    def scatter_device(self, atoms, pix, phys, out=None, accumulate=False, launch=None, _depth=0):
        """Run the configured sum on staged atoms/pixels; float64 (P, 2) on the
        device. When device memory runs out the atoms are summed in halves
        into the same field, down to 1/64 of the sample, as the reference
        retries its chunks (Beam.py:1496-1502); then RuntimeError."""
        try:
            return self._scatter_once(atoms, pix, phys, out, accumulate, launch)
        except (torch.cuda.OutOfMemoryError, MemoryError) as e:
            if _depth >= self.MAX_SPLIT_DEPTH or atoms.n < 2:
                raise RuntimeError("out of device memory even for one kernel chunk") from e
        torch.cuda.empty_cache()
        if out is None:
            out = torch.zeros((pix.n, 2), dtype=torch.float64, device=pix.xyz.device)
            accumulate = True
        half = atoms.n // 2
        for k, sl in enumerate((slice(0, half), slice(half, atoms.n))):
            sp = atoms.species[sl]
            counts = torch.bincount(sp.long(), minlength=len(atoms.table.labels)).cpu().numpy()
            part = engine.Atoms(atoms.pos[sl], sp, atoms.amp[sl], counts.astype(np.int64),
                                atoms.table)
            self.scatter_device(part, pix, phys, out=out, accumulate=accumulate or k > 0,
                                launch=launch, _depth=_depth + 1)
        self.last_run = dict(self.last_run,
                             memory_splits=max(self.last_run.get("memory_splits", 0), _depth + 1))
        return out

    def split_setup(self, tiles, pix, phys=None):
        """What the FP32 split form may do with these tiles and pixels: an
        ``autotune.Setup`` (grouping level, |d|^2 term), or None when the
        geometry leaves the split form's error budget (then the FP64 sum
        runs, as the reference's fast kernel declines to its general kernel,
        Beam.py:1376-1441). Returns (setup or None, diagnostics)."""
        from .autotune import Setup
        third, fresnel, tol, diag = self.split_budget(tiles, pix.r0_min())
        excursion = 2.0 * diag["tile_radius_m"] / max(pix.r0_min(), 1e-30)
        analyser = int(phys.analyser) if phys is not None else 0
        if phys is not None:
            ana_err = self.analyser_budget(tiles, pix.r0_min(), phys)
            if ana_err > 1e-5:
                return None, dict(diag, analyser_err=ana_err,
                                  declined="Darwin analyser varies too fast across a tile")
        if not (third <= tol and excursion < 1e-6):
            return None, dict(diag, declined="split-phase error budget")
        # one sin/cos per pixel pair or 2x2 quad where the geometry allows
        # it; the quad's dropped phase shares the budget with the
        # third-order terms
        level, ginfo = engine.pixel_grouping(tiles, pix, self.k, tol - third,
                                             fresnel_rad=diag["fresnel_rad"] if fresnel else 0.0,
                                             analyser=analyser)
        return Setup(tiles, level, ginfo, int(fresnel), diag["fresnel_radius_m"]), diag

    def tile_atoms_for(self, n_pix, kind="exposure"):
        """Atoms per tile: ``_kernel_tile_atoms`` when set, else the
        autotuner's cached choice for this detector size (512 untuned)."""
        if self._kernel_tile_atoms:
            return int(self._kernel_tile_atoms)
        from . import autotune
        return autotune.tile_atoms(n_pix, kind)

    def choose_split(self, atoms, pix, phys, launch=None):
        """Tiles, set-up and launch shape of the FP32 split sum for these
        atoms and pixels: an explicit ``launch`` or ``_kernel_launch`` (tile
        size ``_kernel_tile_atoms`` or the cached one), else the autotuner's
        cached choice for this detector size, else -- when ``_autotune`` --
        tuned now over tile sizes and launch shapes (the result is cached),
        else the defaults. Returns (setup or None when the geometry declines
        the split form, launch dict, where it came from, diagnostics)."""
        from . import autotune
        explicit = launch or self._kernel_launch
        if not explicit and not phys.analyser and self._autotune and \
                autotune.cached(pix.n) is None:
            sizes = ([int(self._kernel_tile_atoms)] if self._kernel_tile_atoms
                     else list(autotune.TILE_SIZES))
            setups, diags = {}, {}
            for T in sizes:
                su, diag = self.split_setup(engine.Tiles(atoms, self.k, T, device=atoms.pos.device),
                                            pix, phys)
                diags[T] = diag
                if su is not None:
                    setups[T] = su
            if not setups:
                return None, None, "declined", diags[sizes[0]]
            best, self.last_tune = autotune.tune(setups, pix, phys, atoms.table)
            T = int(best.pop("tile_atoms"))
            return setups[T], best, "tuned", diags[T]
        tiles = engine.Tiles(atoms, self.k, self.tile_atoms_for(pix.n), device=atoms.pos.device)
        su, diag = self.split_setup(tiles, pix, phys)
        if su is None:
            return None, None, "declined", diag
        if explicit:
            return su, dict(explicit), "explicit" if launch else "beam", diag
        src = "cached" if autotune.cached(pix.n) is not None else "default"
        return su, tuned_launch(pix.n, su.level, tiles.tile_atoms), src, diag

    def _scatter_once(self, atoms, pix, phys, out=None, accumulate=False, launch=None):
        if self._use_fast_kernel and atoms.n > 0:
            su, cfg, src, diag = self.choose_split(atoms, pix, phys, launch)
            if su is not None:
                tiles = su.tiles
                cfg = engine.grouping_launch(cfg, su.level, tiles, pix, self.k, su.info)
                if phys.analyser:
                    cfg = engine.analyser_launch(cfg)
                res = engine.run_split(tiles, pix, phys, atoms.table, launch=cfg,
                                       fresnel=su.fresnel, out=out, accumulate=accumulate,
                                       fresnel_radius=su.fresnel_radius)
                self.last_run = dict(path="split_f32", n_tiles=tiles.n_tiles,
                                     tile_atoms=tiles.tile_atoms, fresnel=bool(su.fresnel),
                                     factor_table=engine.factor_table_ok(tiles, pix, phys),
                                     launch=dict(cfg), launch_source=src, **su.info, **diag)
                return res
            self.last_run = dict(path="plain_f64", **diag)
        else:
            self.last_run = dict(path="plain_f64")
        return engine.run_plain(atoms, pix, phys, out=out, accumulate=accumulate)

    def interact_beam_gpu(self, sample, measurement_positions, measurement_shape, stage,
                          remove_forward: bool = False, use_depth_ein: bool = False,
                          ein_cache_dir=None, recompute_cache: bool = False,
                          apply_polarization: bool = False, spherical_decay: bool = True,
                          analyser_mode="off", analyser_acceptance_angle_rad: float = 0.0,
                          analyser_darwin_halfwidth_rad: float = 0.0, return_double=False):
        """Kinematic scattering on the GPU (Beam.py:6028-6407); complex (Nz, Ny).

        ``analyser_mode`` "top-hat" / "darwin" (or 1 / 2) applies the general
        kernel's analyser factor (Beam.py:2350-2378) about the axis from the
        origin to the detector's centre pixel (Beam.py:6127-6131)."""
        kind = engine.analyser_kind(analyser_mode)
        if not torch.cuda.is_available():
            raise RuntimeError("interact_beam_gpu: no CUDA GPU (this library has no CPU path)")
        self._require_forward_beam()
        Ny, Nz = int(measurement_shape[0]), int(measurement_shape[1])
        if int(sample.chunk_total or 0) == 0:
            return np.zeros((Nz, Ny), dtype=np.complex128 if return_double else np.complex64)
        coords = np.asarray(measurement_positions)
        if coords.shape != (3, Ny * Nz):
            raise ValueError(f"pixel coordinates {coords.shape} do not match shape ({Ny}, {Nz})")
        analyser = None
        if kind:
            cidx = (Nz // 2) * Ny + (Ny // 2)
            centre = (coords[:, cidx].astype(np.float32) / np.float32(1e10)).astype(np.float64)
            analyser = (kind, centre, float(analyser_acceptance_angle_rad),
                        float(analyser_darwin_halfwidth_rad))
        phys = self.physics(apply_polarization, spherical_decay, remove_forward, analyser=analyser)
        atoms = self.stage_atoms(sample, stage)
        if use_depth_ein:
            # computed on the device for every call; the reference's on-disk
            # cache (ein_cache_dir, recompute_cache) has nothing to save here
            self.apply_depth_ein(atoms)
        pix = self._pixels_for(coords, Ny, Nz, phys)
        out = self.scatter_device(atoms, pix, phys)
        engine.sync()
        field = torch.view_as_complex(out).cpu().numpy().reshape(Nz, Ny)
        return field if return_double else field.astype(np.complex64)

    def _pixels_for(self, coords, Ny, Nz, phys):
        """The prepared pixels of these coordinates and physics: kept from
        the previous call when both are unchanged (a detector is usually
        fixed across exposures), so that their arrays and the pixel-grouping
        bounds derived from them are not rebuilt every call."""
        key = bytes(phys)
        c = self._pix_cache
        if (c is not None and c[1] == (Ny, Nz) and c[2] == key and c[0].shape == coords.shape
                and np.array_equal(c[0], coords)):
            self.last_pixels_cached = True
            return c[3]
        self.last_pixels_cached = False
        pix = engine.Pixels(np.asarray(coords, dtype=np.float64) / 1e10, Ny, Nz, phys)
        self._pix_cache = (np.array(coords, copy=True), (Ny, Nz), key, pix)
        return pix

    def atomic_scattering_kinematic(self, sample, detector, stage, offset=None, use_gpu=True,
                                    remove_forward: bool = False, use_depth_ein: bool = False,
                                    ein_cache_dir=None, recompute_cache: bool = False,
                                    apply_polarization: bool = False,
                                    spherical_decay: bool = False, analyser_mode="off",
                                    analyser_acceptance_angle_rad: float = 0.0,
                                    analyser_darwin_halfwidth_rad: float = 0.0,
                                    return_double: bool = False):
        """Single-bounce kinematic field on the detector (Beam.py:6409-6496):
        complex64 (Nz, Ny) (complex128 with ``return_double``), minus
        ``offset`` when given."""
        if not use_gpu:
            raise RuntimeError("atomic_scattering_kinematic: use_gpu=False is not supported; "
                               "this library runs the sum on the GPU only")
        Ny, Nz = detector.shape
        field = self.interact_beam_gpu(
            sample, detector.pixel_coordinates, (Ny, Nz), stage, remove_forward=remove_forward,
            use_depth_ein=use_depth_ein, ein_cache_dir=ein_cache_dir,
            recompute_cache=recompute_cache, apply_polarization=apply_polarization,
            spherical_decay=spherical_decay, analyser_mode=analyser_mode,
            analyser_acceptance_angle_rad=analyser_acceptance_angle_rad,
            analyser_darwin_halfwidth_rad=analyser_darwin_halfwidth_rad,
            return_double=return_double)
        return (field - offset) if offset is not None else field

    def atomic_direct_interaction(self, sample, detector, stage, scattering=True, sc_kwargs=None,
                                  transmission=False, tr_kwargs=None, use_gpu=True):
        """Scattering term written to the detector (Beam.py:7771-7824)."""
        if transmission:
            raise NotImplementedError("the transmission term is not provided")
        Ny, Nz = detector.shape
        final = np.zeros((Nz, Ny), dtype=np.complex64)
        if scattering:
            final += np.asarray(self.atomic_scattering_kinematic(sample=sample, detector=detector,
                                                                 stage=stage, **(sc_kwargs or {})),
                                dtype=np.complex64)
        detector.input_pixel_values(final)


    # --------------------------------------------------------- propagation
    def wavefield_propagation(self, detector, optics, use_gpu=True, step_max=None, pad_factor=1.0,
                              padding_mode="edge", pad_constant=0.0, save_field=True):
        """Propagate the detector field through an optics stack
        (Beam.py:8024-8095): free-space segments run on the GPU
        (``propagation.propagate``); ``optics`` is a reference optics object
        or a ``propagation.FreeSpaceStack``."""
        from . import propagation
        if not use_gpu:
            raise RuntimeError("wavefield_propagation: use_gpu=False is not supported")
        dy, dz = np.asarray(detector.pixel_size, dtype=np.float64) * 1e-10
        E = detector.pixel_values
        if E is None:
            raise ValueError("detector.pixel_values is None. Run atomic_direct_interaction() first "
                             "to populate the detector field before calling wavefield_propagation().")
        if self._wavelength is None:
            raise ValueError("Beam wavelength is not set. Call create_beam() first.")

        def free_space(F, dym, dzm, z):
            return propagation.propagate(F, dym, dzm, z, self._wavelength, step_max=step_max,
                                         pad_factor=pad_factor, padding_mode=padding_mode,
                                         pad_constant=pad_constant)

        E = optics.apply_stack(field=E, dx=dy, dy=dz, wavelength=self._wavelength,
                               propagate_free_space=free_space, use_gpu=True)
        if isinstance(E, torch.Tensor):
            E = E.cpu().numpy()
        E = np.asarray(E).astype(np.complex64)
        if save_field:
            detector.input_pixel_values(E)
            return None
        return E


def tuned_launch(n_pix, level=0, tile_atoms=None):
    """Launch shape for the split kernel: the autotuner's cached winner for
    this detector size and tile size, or the default when none is cached
    (``level``: 0 no pixel sharing, 1 pairs, 2 quads allowed)."""
    from . import autotune
    return autotune.lookup(n_pix, level, "exposure", tile_atoms)
