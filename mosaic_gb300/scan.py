"""Batched scans: every step of a motor scan in one persistent launch.

The reference runs a scan as one full exposure per step
(experiment.scan_nD, Experiment.py:285-336): reload and re-stage every chunk,
transform the atoms to the lab, sort, plan and launch, per frame. Here the
atoms are staged once, in the SAMPLE frame, and each frame f only changes
what is cheap to change -- its pixels, incident direction and polarization
vector, all moved into the sample frame by the inverse stage transform:

    P'_f = R_f^T (P_f - t_f),   b_f = R_f^T x,   e_f = R_f^T e.

k (b_f . a + |P'_f - a|) is then exactly the phase of atom a at pixel P_f
with the sample at (R_f, t_f). All frames (each with its own ROI, of any
size) become work items of one persistent kernel (``mk_kin_scan_f32``);
the launch sequence can be captured in a CUDA graph and replayed.

The incident amplitude must not depend on the frame: the beam profile must
be uniform and cover the sample in every frame (checked; otherwise run the
frames one by one through ``beam.atomic_scattering_kinematic``).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib, engine
from ._lib import MkFrameDesc, MkLaunch, MkPixels, check


@dataclass
class Frame:
    """One scan step: sample rotation/translation (sample -> lab, A), lab
    pixel coordinates (3, P) in A of its ROI, and the ROI shape (ny, nz)."""
    rotation: np.ndarray
    translation: np.ndarray
    pixels: np.ndarray
    shape: tuple


def roi_indices(det_shape, side, centre=None):
    """Pixel indices (iz*Ny + iy) of a square ROI of ``side`` pixels centred
    on the detector (or on ``centre`` = (iy, iz)), clipped to the detector."""
    ny, nz = int(det_shape[0]), int(det_shape[1])
    sy, sz = min(int(side), ny), min(int(side), nz)
    cy, cz = (ny // 2, nz // 2) if centre is None else centre
    y0 = int(np.clip(cy - sy // 2, 0, ny - sy))
    z0 = int(np.clip(cz - sz // 2, 0, nz - sz))
    iz, iy = np.mgrid[z0:z0 + sz, y0:y0 + sy]
    return (iz * ny + iy).ravel(), (sy, sz)


class BatchedScan:
    """All frames of a scan as one launch over atoms staged once.

    Args:
        beam: a configured ``mosaic_gb300.beam``.
        sample: chunk-API sample (thermal displacement applied on load).
        frames: list of Frame.
        apply_polarization, spherical_decay, remove_forward: as in
            ``atomic_scattering_kinematic``.
        launch: split-kernel launch shape (None: the beam's ``_kernel_launch``,
            else the autotuner's cached choice for this scan size, else tuned
            now on a probe of the first frames when ``tune`` (default: the
            beam's ``_autotune``), else the default).
        staged: an earlier BatchedScan of the same sample whose atoms and
            tiles this one reuses.
    """

    def __init__(self, beam, sample, frames, apply_polarization=False, spherical_decay=False,
                 remove_forward=False, launch=None, device="cuda", staged=None, tune=None):
        self.L = engine._require_cuda()
        self.beam = beam
        self.frames = list(frames)
        if not self.frames:
            raise ValueError("a scan needs at least one frame")
        beam._require_forward_beam()
        dev = torch.device(device)
        self._dev = dev
        self._flags = dict(apply_polarization=apply_polarization, spherical_decay=spherical_decay,
                           remove_forward=remove_forward)
        pol = beam._polarization_state()
        e_lab = np.array(pol[1:4], dtype=np.float64)
        b_lab = np.array([1.0, 0.0, 0.0])
        xyz, fr, bdirs, pols = [], [], [], []
        for f in self.frames:
            R = np.asarray(f.rotation, dtype=np.float64)
            t = np.asarray(f.translation, dtype=np.float64)
            P = np.asarray(f.pixels, dtype=np.float64)
            xyz.append((R.T @ (P - t[:, None])) / 1e10)
            b = R.T @ b_lab
            fr.append((int(f.shape[0]), int(f.shape[1]), b))
            bdirs.append(b)
            pols.append(R.T @ e_lab)
        self.frame_pixels = np.array([int(s[0]) * int(s[1]) for s in fr], dtype=np.int32)
        self.frame_rows = np.array([int(s[0]) for s in fr], dtype=np.int32)
        self.offsets = np.concatenate([[0], np.cumsum(self.frame_pixels)]).astype(np.int64)
        n_total = int(self.offsets[-1])
        self._bd = np.ascontiguousarray(np.array(bdirs, dtype=np.float64))
        self._pe = np.ascontiguousarray(np.array(pols, dtype=np.float64))
        self._staged = staged is not None
        if staged is not None:
            # reuse the atoms and tiles of an earlier scan of the same sample
            self._rmax = staged._rmax
            self._check_uniform_beam(None)
            self.atoms, self.table, self.tiles = staged.atoms, staged.table, staged.tiles
        else:
            pos, idx, labels = beam.collect_atoms(sample)
            self._rmax = (float(np.sqrt((pos.astype(np.float64) ** 2).sum(1)).max())
                          if pos.shape[0] else 0.0)
            self._check_uniform_beam(None)
            table = engine.SpeciesTable.build(labels or ["H"], beam.tables, beam._energy,
                                              beam._debye_waller)
            # atoms in the sample frame, incident amplitude 1
            self.atoms = engine.atoms_lab(pos, idx, np.eye(3), np.zeros(3), table, device=dev)
            self.table = table
            self.tiles = engine.Tiles(self.atoms, beam.k, beam.tile_atoms_for(n_total, "scan"),
                                      device=dev)
        self.phys = beam.physics(apply_polarization, spherical_decay, remove_forward, pol=pol)
        self.pix = engine.Pixels(np.concatenate(xyz, axis=1), n_total, 1, self.phys, device=dev,
                                 frames=fr)
        su = self._setup(self.tiles)
        self.tune_results = []
        if launch:
            cfg, src = dict(engine.default_launch(su.level, self.tiles.tile_atoms), **launch), "explicit"
        elif beam._kernel_launch:
            cfg, src = dict(engine.default_launch(su.level, self.tiles.tile_atoms),
                            **beam._kernel_launch), "beam"
        else:
            from . import autotune
            best = autotune.cached(n_total, "scan")
            src = "cached" if best else "default"
            if tune is None:
                tune = beam._autotune
            if best is None and tune and len(self.frames) > 1:
                best, self.tune_results = autotune.tune_scan(self, self._setups(su))
                src = "tuned"
            if best and not self._staged and \
                    int(best.get("tile_atoms", self.tiles.tile_atoms)) != self.tiles.tile_atoms:
                tiles = engine.Tiles(self.atoms, beam.k, int(best["tile_atoms"]), device=dev)
                try:
                    su, self.tiles = self._setup(tiles), tiles
                except _lib.DeclineError:
                    pass
            cfg = (autotune.lookup(n_total, su.level, "scan", self.tiles.tile_atoms) if best
                   else engine.default_launch(su.level, self.tiles.tile_atoms))
        self.launch_source = src
        self.out = torch.zeros((n_total, 2), dtype=torch.float64, device=dev)
        self.sums = torch.zeros(len(self.frames), dtype=torch.float64, device=dev)
        self.ws, self.ws_bytes = None, 0
        self.replan(self.tiles, su, cfg)
        self.terms = float(self.atoms.n) * n_total

    def _setup(self, tiles):
        """The split form's set-up for these tiles (raises when the scan's
        geometry leaves its error budget)."""
        su, diag = self.beam.split_setup(tiles, self.pix)
        if su is None:
            raise _lib.DeclineError(_lib.MK_EDECLINE,
                                    f"scan geometry outside the split-phase error budget "
                                    f"({diag.get('declined', '')}; third-order "
                                    f"{diag['third_order_rad']:.2e} rad)")
        self.diag = dict(diag, **su.info)
        return su

    def _setups(self, su):
        """{atoms per tile: Setup} the tuner tries: the scan's own tiles and,
        unless they are shared with another scan, the other tile sizes."""
        from . import autotune
        out = {self.tiles.tile_atoms: su}
        if self._staged:
            return out
        for T in autotune.TILE_SIZES:
            if T in out:
                continue
            t = engine.Tiles(self.atoms, self.beam.k, T, device=self._dev)
            s2, _ = self.beam.split_setup(t, self.pix)
            if s2 is not None:
                out[T] = s2
        self.diag = dict(self.diag)
        return out

    def probe(self, n_frames, launch=None):
        """A scan of this scan's first ``n_frames`` frames over the same
        staged atoms (the autotuner's probe; also a cheap warm-up of a
        launch shape before a long scan is captured)."""
        return BatchedScan(self.beam, None, self.frames[:n_frames], staged=self, tune=False,
                           launch=launch or engine.default_launch(0), device=self._dev,
                           **self._flags)

    def replan(self, tiles, su, cfg):
        """Plan the launch for ``tiles`` (this scan's, or a view of them) with
        launch dict ``cfg`` (clamped to what ``su`` allows)."""
        cfg = engine.grouping_launch(cfg, su.level, tiles, self.pix, self.beam.k, su.info)
        self.cfg = cfg
        self.setup = su
        self.tiles_run = tiles
        self.launch = MkLaunch(int(cfg["pix_per_thread"]), int(cfg["threads"]), int(cfg["slices"]),
                               int(su.fresnel), int(tiles.amp_is_real()), float(su.fresnel_radius),
                               int(cfg["pairs"]), float(cfg["pair_short_radius_m"]),
                               float(cfg.get("sin_direct_max_rad", 0.0) or 0.0),
                               float(cfg.get("octet_radius_m", 0.0) or 0.0))
        nf = len(self.frames)
        desc = (MkFrameDesc * nf)()
        n_items, n_part = ctypes.c_longlong(0), ctypes.c_longlong(0)
        check(self.L.mk_scan_plan(nf, self.frame_pixels.ctypes.data, self.frame_rows.ctypes.data,
                                  self._bd.ctypes.data, self._pe.ctypes.data,
                                  ctypes.byref(tiles.abi), ctypes.byref(self.launch),
                                  ctypes.cast(desc, ctypes.c_void_p), ctypes.byref(n_items),
                                  ctypes.byref(n_part)))
        self.n_items, self.n_partial = int(n_items.value), int(n_part.value)
        raw = np.frombuffer(bytes(desc), dtype=np.uint8).copy()
        self.frames_dev = torch.as_tensor(raw).to(self._dev)
        # per-(species, pixel) factors at every frame's pixel directions,
        # where the tile origins allow it (engine.factor_table_ok)
        self.pix_abi, self.ftab = self.pix.abi, None
        if engine.factor_table_ok(tiles, self.pix, self.phys):
            key = (self.table.key(), bytes(raw))
            if getattr(self, "_ftab_key", None) == key and self._ftab is not None:
                self.ftab = self._ftab
            else:
                self.ftab = torch.empty((len(self.table.labels), self.pix.n, 2),
                                        dtype=torch.float32, device=self._dev)
                abi = MkPixels.from_buffer_copy(self.pix.abi)
                abi.factor = self.ftab.data_ptr()
                sp = self.table.abi()
                check(self.L.mk_factor_table(ctypes.byref(abi), ctypes.byref(sp),
                                             ctypes.byref(self.phys), nf,
                                             self.frames_dev.data_ptr(), engine._stream_handle()))
                self._ftab_key, self._ftab = key, self.ftab
            self.pix_abi = MkPixels.from_buffer_copy(self.pix.abi)
            self.pix_abi.factor = self.ftab.data_ptr()
        need = int(self.L.mk_scan_workspace_size(self.n_partial))
        if self.ws is None or self.ws_bytes < need:
            self.ws = torch.empty(need, dtype=torch.uint8, device=self._dev)
            self.ws_bytes = need
        self._graph = None

    def _check_uniform_beam(self, pos):
        B = self.beam
        if not str(B._beam_profile).startswith("uniform") and B._beam_profile != "uniform":
            raise NotImplementedError("batched scans need a uniform beam profile; run the frames "
                                      "one by one through atomic_scattering_kinematic")
        if not np.all(np.abs(B._beam_E0_map) == 1.0):
            raise NotImplementedError("batched scans need a uniform beam map")
        if self._rmax > 0.0:
            rmax = self._rmax
            for f in self.frames:
                c = np.asarray(f.translation, dtype=np.float64)
                half_u = 0.5 * B._beam_size[0] - abs(c[1])
                half_v = 0.5 * B._beam_size[1] - abs(c[2])
                if rmax >= min(half_u, half_v) - max(B._beam_du, B._beam_dv):
                    raise NotImplementedError(
                        "the beam does not cover the sample in every frame; batched scans need "
                        "a frame-independent incident amplitude")

    def run(self, stream=None):
        """Launch the whole scan (asynchronous); returns (fields, sums) on device."""
        sp = self.table.abi()
        check(self.L.mk_kin_scan_f32(ctypes.byref(self.tiles_run.abi), ctypes.byref(sp),
                                     ctypes.byref(self.phys), ctypes.byref(self.pix_abi),
                                     len(self.frames), self.frames_dev.data_ptr(), self.n_items,
                                     self.n_partial, ctypes.byref(self.launch), self.out.data_ptr(),
                                     self.sums.data_ptr(), self.ws.data_ptr(), self.ws_bytes,
                                     engine._stream_handle(stream)))
        return self.out, self.sums

    def capture(self, warm=True):
        """Capture run() in a CUDA graph (frames > 1); replay() then re-runs it.
        ``warm`` runs the scan once outside the capture first (the kernels'
        first-use set-up); a caller that has already run a scan with the same
        launch shape (a short one, e.g.) may skip it."""
        if len(self.frames) < 2:
            raise ValueError("graph capture needs at least two frames")
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        if warm:
            with torch.cuda.stream(s):
                self.run(s)             # warm-up outside the capture
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run(torch.cuda.current_stream())
        self._graph = g
        return g

    def replay(self):
        if self._graph is None:
            self.capture()
        self._graph.replay()
        return self.out, self.sums

    def frame_field(self, f):
        """Complex128 (nz, ny) field of frame f (host)."""
        ny, nz = self.frames[f].shape
        a, b = int(self.offsets[f]), int(self.offsets[f + 1])
        return torch.view_as_complex(self.out[a:b]).cpu().numpy().reshape(int(nz), int(ny))

    def sum_intensity(self):
        return self.sums.cpu().numpy()


def frames_from_motors(stage, detector, steps, rois=None):
    """Frames for a list of motor settings.

    steps: list of dicts {motor name: value (radians for rotations, A for
    translations)} applied to ``stage`` (restored afterwards); ``rois``:
    per-step ROI side (int) or None for the full detector."""
    saved = stage._motor_value.copy()
    out = []
    try:
        for i, st in enumerate(steps):
            stage._motor_value[:] = saved
            for name, v in st.items():
                stage._motor_value[stage.motor_index(name)] = float(v)
            R, t = stage.get_rotation().copy(), stage.get_translation().copy()
            coords = np.asarray(detector.pixel_coordinates)
            if rois is not None and rois[i] is not None:
                sel, shape = roi_indices(detector.shape, rois[i])
                coords = coords[:, sel]
            else:
                shape = tuple(detector.shape)
            out.append(Frame(R, t, coords, shape))
    finally:
        stage._motor_value[:] = saved
        stage.get_rotation()
        stage.get_translation()
    return out
