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


CONFIGS = {"fcc_cu_32k": fcc_cu_32k, "nacl_screw_8m": nacl_screw_8m}


def build(name, **kw):
    return CONFIGS[name](**kw)
