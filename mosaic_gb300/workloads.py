"""Seeded synthetic workloads with the shapes of the benchmark configurations.

There is no public dataset on this path: the reference builds its samples
from CIF files and defect models (outside this library). These generators
produce the same kinds of samples directly, seeded and reproducible:

* ``fcc_cu_32k``: fcc Cu (a = 3.615 A), 20^3 cells = 32,000 atoms, Gaussian
  thermal displacement sigma = 0.08 A (seed 40, clip 1 A) by the reference's
  rule, 10 keV, sigma-polarised, 128 x 128 pixels of 55 um at 1.0 m centred on
  the Cu (111) Bragg condition; [111] along the sample z axis and the stage mu
  motor at theta_B puts G_111 along the scattering vector.
* ``nacl_screw_8m``: rocksalt Na/Cl (a = 5.64 A), 160 x 160 x 40 cells =
  8,192,000 atoms in 16 chunks (4 x 4 columns of 40^3 cells), screw
  dislocation along [001] through the centre, u_z = b/(2 pi) atan2(y, x),
  b = 3.99 A; 512 x 512 pixels at the (002) reflection (G parallel to the
  line, so g.b != 0), 10 keV, 1.0 m, 55 um, sigma-polarised.

Unstated parameters of the configurations (energy, distance and pitch of the
rocksalt case) are fixed here and recorded in each workload's ``meta``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .beam import beam as Beam
from .geometry import Detector, Stage, align_rotation
from .sample import ChunkedSample

HC_EV_A = 12398.419843320026   # h c / e in eV A


def bragg_theta(d_A, energy_eV):
    return float(np.arcsin((HC_EV_A / energy_eV) / (2.0 * d_A)))


def fcc_basis():
    return np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]], dtype=np.float64)


def lattice(a, cells, basis):
    """(prod(cells)*len(basis), 3) float64 positions, cell-major order."""
    nx, ny, nz = cells
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1)
    g = g.reshape(-1, 1, 3).astype(np.float64)
    return ((g + basis[None]) * a).reshape(-1, 3)


@dataclass
class Workload:
    name: str
    sample: object
    detector: Detector
    stage: Stage
    beam: Beam
    sc_kwargs: dict
    meta: dict = field(default_factory=dict)

    @property
    def n_atoms(self):
        return self.sample.n_atoms

    @property
    def n_pixels(self):
        return int(self.detector.shape[0]) * int(self.detector.shape[1])

    @property
    def terms(self):
        return float(self.n_atoms) * self.n_pixels


def _detector(shape, pitch_A, distance_A, two_theta_rad, eta_rad=0.0):
    D = Detector()
    D.create_detector(shape, (pitch_A, pitch_A))
    D.position_detector_absolute(distance_A, two_theta_rad, eta_rad, degrees=False)
    return D


def _beam(energy, size_A, pol_perp_rate=1.0):
    B = Beam()
    B.create_beam(energy, beam_size=(size_A, size_A), beam_samples=(256, 256),
                  pol_perp_rate=pol_perp_rate)
    return B


def fcc_cu_32k(cells=20, npix=128, thermal=True):
    a, E = 3.615, 10000.0
    pos = lattice(a, (cells,) * 3, fcc_basis())
    pos -= pos.mean(axis=0)
    pos = pos @ align_rotation([1, 1, 1], [0, 0, 1]).T
    spc = np.full(pos.shape[0], "Cu")
    th = dict(sigma=0.08, max_displacement=1.0, seed=40) if thermal else None
    sample = ChunkedSample([(pos.astype(np.float32), spc)], thermal=th)
    theta = bragg_theta(a / np.sqrt(3.0), E)
    det = _detector((npix, npix), 5.5e5, 1.0e10, 2 * theta)
    st = Stage()
    st.set_motor_value("mu", theta, degrees=False)
    diag = float(np.linalg.norm(pos.max(0) - pos.min(0)))
    B = _beam(E, max(1000.0, 2.5 * diag))
    return Workload("fcc_cu_32k", sample, det, st, B,
                    dict(apply_polarization=True, spherical_decay=False, remove_forward=False),
                    dict(a=a, energy_eV=E, theta_deg=np.degrees(theta), cells=cells, npix=npix,
                         distance_m=1.0, pitch_um=55.0, thermal_sigma_A=0.08 if thermal else 0.0))


def nacl_screw_8m(cells=(160, 160, 40), npix=512, chunk_grid=(4, 4), b_A=3.99):
    a, E = 5.64, 10000.0
    basis_na = fcc_basis()
    basis_cl = basis_na + np.array([0.5, 0.0, 0.0])
    nx, ny, nz = cells
    cx, cy = nx // chunk_grid[0], ny // chunk_grid[1]
    centre = 0.5 * a * np.array([nx, ny, nz], dtype=np.float64)
    chunks = []
    for i in range(chunk_grid[0]):
        for j in range(chunk_grid[1]):
            off = np.array([i * cx, j * cy, 0]) * a
            na = lattice(a, (cx, cy, nz), basis_na) + off
            cl = lattice(a, (cx, cy, nz), basis_cl) + off
            pos = np.concatenate([na, cl]) - centre
            pos[:, 2] += (b_A / (2 * np.pi)) * np.arctan2(pos[:, 1], pos[:, 0])
            codes = np.concatenate([np.zeros(len(na), np.uint8), np.ones(len(cl), np.uint8)])
            chunks.append((pos.astype(np.float32), (codes, np.array(["Na", "Cl"]))))
    sample = ChunkedSample(chunks)
    theta = bragg_theta(a / 2.0, E)
    det = _detector((npix, npix), 5.5e5, 1.0e10, 2 * theta)
    st = Stage()
    st.set_motor_value("mu", theta, degrees=False)
    diag = float(np.linalg.norm(centre * 2))
    B = _beam(E, max(1000.0, 2.5 * diag))
    return Workload("nacl_screw_8m", sample, det, st, B,
                    dict(apply_polarization=True, spherical_decay=False, remove_forward=False),
                    dict(a=a, energy_eV=E, theta_deg=np.degrees(theta), cells=list(cells),
                         npix=npix, distance_m=1.0, pitch_um=55.0, burgers_A=b_A,
                         reflection="(002), G parallel to the dislocation line"))


def random_rotations(n, rng):
    """n rotation matrices uniform on SO(3) (unit quaternions, Shoemake)."""
    u1, u2, u3 = rng.random((3, n))
    q = np.stack([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)], 1)
    x, y, z, w = q.T
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], 1),
                     np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], 1),
                     np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], 1)], 1)


def polycrystal_positions(box_A=600.0, n_grains=64, a=3.615, seed=2026, voxel_A=10.0,
                          stacking_fault=True, device=None):
    """Voronoi polycrystal of fcc grains filling a cube of side ``box_A``
    centred on 0. Each grain: seeded centre, uniformly random orientation,
    and (optionally) one intrinsic stacking fault -- the atoms on the far
    side of the grain's (111) plane through its centre shifted by
    (a/6)[1 1 -2] in the grain frame. Returns (N, 3) float32 and the grain id
    per atom. Runs on the GPU through torch when ``device`` is a CUDA device."""
    import torch
    rng = np.random.default_rng(seed)
    half = box_A / 2.0
    seeds = rng.random((n_grains, 3)) * box_A - half
    rots = random_rotations(n_grains, rng)
    dev = torch.device(device) if device is not None else torch.device("cpu")
    S = torch.tensor(seeds, dtype=torch.float64, device=dev)
    nv = int(np.ceil(box_A / voxel_A))
    g1 = (torch.arange(nv, dtype=torch.float64, device=dev) + 0.5) * (box_A / nv) - half
    V = torch.stack(torch.meshgrid(g1, g1, g1, indexing="ij"), -1).reshape(-1, 3)
    lab = torch.cdist(V, S).argmin(1)
    basis = torch.tensor(fcc_basis(), dtype=torch.float64, device=dev)
    out_pos, out_gid = [], []
    margin = 2.0 * voxel_A
    for g in range(n_grains):
        Vg = V[lab == g]
        if Vg.shape[0] == 0:
            continue
        lo = torch.clamp(Vg.min(0).values - margin, min=-half)
        hi = torch.clamp(Vg.max(0).values + margin, max=half)
        Rg = torch.tensor(rots[g], dtype=torch.float64, device=dev)
        c = S[g]
        corners = torch.stack([torch.stack([x, y, z]) for x in (lo[0], hi[0])
                               for y in (lo[1], hi[1]) for z in (lo[2], hi[2])])
        loc = (corners - c) @ Rg / a                      # grain-frame lattice coordinates
        n0 = torch.floor(loc.min(0).values).long() - 1
        n1 = torch.ceil(loc.max(0).values).long() + 1
        rngs = [torch.arange(int(n0[i]), int(n1[i]) + 1, device=dev, dtype=torch.float64) for i in range(3)]
        cells = torch.stack(torch.meshgrid(*rngs, indexing="ij"), -1).reshape(-1, 1, 3)
        local = ((cells + basis[None]) * a).reshape(-1, 3)
        x = local @ Rg.T + c
        keep = ((x >= lo) & (x <= hi)).all(1)
        x, local = x[keep], local[keep]
        keep = torch.cdist(x, S).argmin(1) == g
        x, local = x[keep], local[keep]
        if stacking_fault:
            nrm = torch.tensor([1.0, 1.0, 1.0], dtype=torch.float64, device=dev) / np.sqrt(3.0)
            side = (local @ nrm) > 0
            shift = torch.tensor([1.0, 1.0, -2.0], dtype=torch.float64, device=dev) * (a / 6.0)
            x = x + side[:, None].double() * (Rg @ shift)[None]
        out_pos.append(x.float().cpu().numpy())
        out_gid.append(np.full(x.shape[0], g, dtype=np.int32))
    return np.concatenate(out_pos), np.concatenate(out_gid)


def cu_polycrystal_18m(box_A=600.0, n_grains=64, npix=1024, chunk_atoms=1_000_000, device=None,
                       seed=2026):
    """Large chunked polycrystal: 64 Voronoi fcc Cu grains in a 60 nm cube
    (~18.3M atoms) in 1M-atom chunks, one stacking fault per grain; 1024^2
    pixels at 0.5 m, 12 keV, centred at Cu(111)."""
    a, E = 3.615, 12000.0
    pos, gid = polycrystal_positions(box_A, n_grains, a, seed, device=device)
    chunks = [(pos[i:i + chunk_atoms], (np.zeros(min(chunk_atoms, pos.shape[0] - i), np.uint8),
                                        np.array(["Cu"])))
              for i in range(0, pos.shape[0], chunk_atoms)]
    sample = ChunkedSample(chunks, dimensions=(box_A,) * 3)
    theta = bragg_theta(a / np.sqrt(3.0), E)
    det = _detector((npix, npix), 5.5e5, 0.5e10, 2 * theta)
    B = _beam(E, 2.5 * box_A * np.sqrt(3.0))
    return Workload("cu_polycrystal_18m", sample, det, Stage(), B,
                    dict(apply_polarization=True, spherical_decay=False, remove_forward=False),
                    dict(a=a, energy_eV=E, theta_deg=np.degrees(theta), grains=n_grains,
                         box_A=box_A, npix=npix, distance_m=0.5, pitch_um=55.0, seed=seed,
                         stacking_fault="(a/6)[1 1 -2] beyond the grain's (111) plane"))


def bump_field_crystal(cells=100, a=3.615, n_bumps=8, amp_A=0.3, width_A=50.0, seed=4):
    """fcc Cu, [111] along z, displaced by a smooth field
    u(r) = sum_b amp n_b exp(-|r - c_b|^2 / (2 width^2)), seeded centres
    (uniform in the crystal) and unit directions."""
    rng = np.random.default_rng(seed)
    pos = lattice(a, (cells,) * 3, fcc_basis())
    pos -= pos.mean(axis=0)
    half = 0.5 * cells * a
    centres = rng.random((n_bumps, 3)) * 2 * half - half
    dirs = rng.standard_normal((n_bumps, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    u = np.zeros_like(pos)
    for c, n in zip(centres, dirs):
        r2 = ((pos - c) ** 2).sum(1)
        u += amp_A * np.exp(-r2 / (2 * width_A ** 2))[:, None] * n[None]
    pos = (pos + u) @ align_rotation([1, 1, 1], [0, 0, 1]).T
    return pos.astype(np.float32), dict(centres=centres.tolist(), dirs=dirs.tolist(), seed=seed)


def rocking_frames(theta_b, n_theta=181, half_range_deg=0.5, chi_offsets_deg=(-0.3, -0.1, 0.1, 0.3),
                   roi_sides=(64, 128, 256, 512)):
    """Frames of the rocking scan: mu = theta_B + dtheta (n_theta steps over
    +-half_range) for every chi offset; ROI side cycles through roi_sides by
    frame index."""
    frames = []
    for ci, chi in enumerate(chi_offsets_deg):
        for ti in range(n_theta):
            dth = -half_range_deg + ti * (2 * half_range_deg / (n_theta - 1))
            f = len(frames)
            frames.append(dict(mu=float(theta_b + np.radians(dth)), chi=float(np.radians(chi)),
                               roi=int(roi_sides[f % len(roi_sides)])))
    return frames


def cu_bumps_scan_4m(cells=100, npix=512, n_theta=181, chi_offsets_deg=(-0.3, -0.1, 0.1, 0.3),
                     roi_sides=(64, 128, 256, 512)):
    """Batched scan: 4M-atom bump-field crystal, rocking scan of n_theta
    steps over +-0.5 deg times the chi offsets, uneven ROIs."""
    a, E = 3.615, 10000.0
    pos, meta = bump_field_crystal(cells, a)
    sample = ChunkedSample([(pos, (np.zeros(pos.shape[0], np.uint8), np.array(["Cu"])))])
    theta = bragg_theta(a / np.sqrt(3.0), E)
    det = _detector((npix, npix), 5.5e5, 1.0e10, 2 * theta)
    st = Stage()
    st.set_motor_value("mu", theta, degrees=False)
    diag = float(np.linalg.norm(pos.max(0) - pos.min(0)))
    B = _beam(E, max(1000.0, 2.5 * diag))
    frames = rocking_frames(theta, n_theta, 0.5, chi_offsets_deg, roi_sides)
    return Workload("cu_bumps_scan_4m", sample, det, st, B,
                    dict(apply_polarization=True, spherical_decay=False, remove_forward=False),
                    dict(a=a, energy_eV=E, theta_deg=np.degrees(theta), cells=cells, npix=npix,
                         distance_m=1.0, pitch_um=55.0, frames=frames,
                         chi_offsets_deg=list(chi_offsets_deg), roi_sides=list(roi_sides), **meta))


def cu_bumps_surrogate_4m(cells=100, npix=512, n_grid=101, half_range_deg=0.3, roi=128):
    """Surrogate scan: the same 4M-atom bump-field crystal, a theta x chi grid
    of n_grid x n_grid frames over +-half_range_deg on each motor (offsets
    from the (111) Bragg setting), a roi x roi ROI at the detector centre."""
    w = cu_bumps_scan_4m(cells=cells, npix=npix)
    grid = np.radians(np.linspace(-half_range_deg, half_range_deg, n_grid))
    w.name = "cu_bumps_surrogate_4m"
    w.meta.update(theta_offsets=grid, chi_offsets=grid.copy(), roi=int(roi),
                  grid=f"{n_grid}x{n_grid} over +-{half_range_deg} deg")
    return w


def nacl_screw_2m():
    """Quarter-size precision case (80 x 80 x 40 cells = 2,048,000 atoms, 256^2
    pixels) for kernel profiles: the same per-term work as nacl_screw_8m."""
    w = nacl_screw_8m(cells=(80, 80, 40), npix=256, chunk_grid=(2, 2))
    w.name = "nacl_screw_2m"
    return w


def nacl_screw_8m_px128():
    """The headline crystal (8,192,000 atoms) on a 128 x 128 detector: a
    profile case whose tiles (~200 MB) exceed L2 like the full run's, so its
    DRAM traffic per pixel block is the full run's."""
    w = nacl_screw_8m(npix=128)
    w.name = "nacl_screw_8m_px128"
    return w


def spread_pixels(det_shape, n=32):
    """Pixel indices (iz * Ny + iy) spread over the whole detector for
    accuracy checks: an n x n grid of rows and columns from edge to edge
    (the four corners included), plus the midpoints of the four edges and
    the centre pixel. n = 32 gives 1,029 pixels."""
    ny, nz = int(det_shape[0]), int(det_shape[1])
    ys = np.unique(np.rint(np.linspace(0, ny - 1, min(n, ny))).astype(np.int64))
    zs = np.unique(np.rint(np.linspace(0, nz - 1, min(n, nz))).astype(np.int64))
    iz, iy = np.meshgrid(zs, ys, indexing="ij")
    pts = set(zip(iz.ravel().tolist(), iy.ravel().tolist()))
    my, mz = ny // 2, nz // 2
    pts |= {(0, my), (nz - 1, my), (mz, 0), (mz, ny - 1), (mz, my)}
    pts = sorted(pts)
    return np.array([z * ny + y for z, y in pts], dtype=np.int64)


CONFIGS = {"fcc_cu_32k": fcc_cu_32k, "nacl_screw_8m": nacl_screw_8m, "nacl_screw_2m": nacl_screw_2m,
           "nacl_screw_8m_px128": nacl_screw_8m_px128,
           "cu_polycrystal_18m": cu_polycrystal_18m, "cu_bumps_scan_4m": cu_bumps_scan_4m,
           "cu_bumps_surrogate_4m": cu_bumps_surrogate_4m}


def build(name, **kw):
    return CONFIGS[name](**kw)
