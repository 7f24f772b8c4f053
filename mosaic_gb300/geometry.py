"""Detector, stage and polarization geometry: the objects the scattering
entry point reads.

These mirror the reference duck types so that either the reference's own
objects or these can be passed to :meth:`mosaic_gb300.beam.atomic_scattering_kinematic`:

* ``Detector``: ``pixel_coordinates`` (3, Ny*Nz) in Angstrom (pixel index
  ``iz*Ny + iy``), ``shape`` (Ny, Nz), ``pixel_size``, ``input_pixel_values``,
  ``pixel_values``, ``pixel_intensity`` (MOSAIC Detector.py:73-313, 620-770,
  1632-1722). Rectangular pixel grids in "plane" or "shell" construction.
* ``Stage``: motor stack with couplings, ``rotation`` (3,3) float32 and
  ``translation`` (3,) float32 (Stage.py:74-160, 252-382).
* ``polarization_from_rate`` / ``polarization_state`` (Beam.py:31-47, 117-149).

Array dtypes follow the reference (float32 base grids and stage matrices,
float64 positioned pixel coordinates), so the same inputs reach the kernels.
"""
from __future__ import annotations

import numpy as np


def polarization_from_rate(rho):
    """(p, ex, ey, ez) for a +x beam from the perpendicular fraction rho."""
    rho = float(np.clip(rho, 0.0, 1.0))
    p = abs(2.0 * rho - 1.0)
    return (p, 0.0, 1.0, 0.0) if rho >= 0.5 else (p, 0.0, 0.0, 1.0)


def polarization_state(pol_perp_rate=0.5, pol_direction=None, pol_degree=None,
                       direction=(1.0, 0.0, 0.0)):
    """Degree p and unit vector e of the linear polarization, e normal to the
    beam; falls back to a transverse lab axis when e lies along the beam."""
    khat = np.asarray(direction, dtype=np.float64)
    khat = khat / np.linalg.norm(khat)
    p_rate, ex, ey, ez = polarization_from_rate(pol_perp_rate)
    p = p_rate if pol_degree is None else float(np.clip(pol_degree, 0.0, 1.0))
    e = (np.array([ex, ey, ez]) if pol_direction is None
         else np.asarray(pol_direction, dtype=np.float64).reshape(3))
    e = e - np.dot(e, khat) * khat
    if np.linalg.norm(e) < 1e-12:
        for ax in (np.array([0.0, 1.0, 0.0]), np.array([0.0, 0.0, 1.0])):
            e = ax - np.dot(ax, khat) * khat
            if np.linalg.norm(e) >= 1e-12:
                break
    e = e / np.linalg.norm(e)
    return float(p), float(e[0]), float(e[1]), float(e[2])


def axis_rotation(axis, angle, dtype=np.float64):
    """Right-handed rotation by ``angle`` (rad) about ``axis`` (Rodrigues)."""
    a = np.asarray(axis, dtype=np.float64)
    x, y, z = a / np.linalg.norm(a)
    c, s = np.cos(angle), np.sin(angle)
    d = 1.0 - c
    return np.array([[c + d * x * x, d * x * y - z * s, d * x * z + y * s],
                     [d * y * x + z * s, c + d * y * y, d * y * z - x * s],
                     [d * z * x - y * s, d * z * y + x * s, c + d * z * z]], dtype=dtype)


def align_rotation(a, b):
    """Rotation (float64) taking unit vector ``a`` onto unit vector ``b``."""
    a = np.asarray(a, float) / np.linalg.norm(a)
    b = np.asarray(b, float) / np.linalg.norm(b)
    v = np.cross(a, b)
    s, c = np.linalg.norm(v), float(np.dot(a, b))
    if s < 1e-15:
        if c > 0:
            return np.eye(3)
        perp = np.cross(a, [1.0, 0.0, 0.0])
        if np.linalg.norm(perp) < 1e-6:
            perp = np.cross(a, [0.0, 1.0, 0.0])
        return axis_rotation(perp, np.pi)
    return axis_rotation(v, np.arctan2(s, c))


class Detector:
    """Rectangular pixel detector (spatial input, plane or shell construction)."""

    def __init__(self):
        self._shape = None
        self._pixel_size = None
        self._pixel_coordinates = None
        self._pixel_values = None
        self._pixel_intensity = None
        self._two_theta = 0.0
        self._eta = 0.0
        self._distance = 0.0
        self._center = np.zeros(3)
        self._direction = np.array([1.0, 0.0, 0.0])
        self._construction_mode = "plane"

    def create_detector(self, shape, pixel_size, geometry="rectangular",
                        construction_mode="plane", input_mode="spatial"):
        """Base grid in the x = 0 plane, pixel centres at pitch ``pixel_size``
        (A), centred on 0 (Detector.py:204-214)."""
        if str(geometry).lower() != "rectangular" or str(input_mode).lower() != "spatial":
            raise NotImplementedError("only rectangular, spatial-input detectors are provided")
        mode = str(construction_mode).lower()
        if mode not in ("plane", "shell"):
            raise ValueError(f"construction_mode must be 'plane' or 'shell', got '{construction_mode}'")
        self._construction_mode = mode
        self._shape = (int(shape[0]), int(shape[1]))
        self._pixel_size = pixel_size
        ny, nz = self._shape
        y = ((np.arange(ny) - (ny - 1) / 2.0) * float(pixel_size[0])).astype(np.float32)
        z = ((np.arange(nz) - (nz - 1) / 2.0) * float(pixel_size[1])).astype(np.float32)
        Y, Z = np.meshgrid(y, z)
        X = np.full_like(Y, 0)
        self._pixel_coordinates = np.vstack((X.ravel(), Y.ravel(), Z.ravel()))
        self._center = np.zeros(3)
        self._direction = np.array([1.0, 0.0, 0.0])

    @staticmethod
    def get_rotation_detector(two_theta, eta):
        """R_eta(-x) @ R_2theta(-y), sending +x to (cos2t, sin2t sin eta, sin2t cos eta)."""
        return axis_rotation([-1.0, 0.0, 0.0], eta) @ axis_rotation([0.0, -1.0, 0.0], two_theta)

    def position_detector_absolute(self, distance, two_theta, eta, degrees=True):
        """Rebuild the base grid, rotate it and centre it at
        distance * (cos 2theta, sin 2theta sin eta, sin 2theta cos eta)
        (Detector.py:620-717)."""
        if self._shape is None:
            raise ValueError("Detector shape/pixel_size are not initialized. "
                             "Call create_detector(...) before positioning.")
        if degrees:
            two_theta, eta = np.deg2rad(two_theta), np.deg2rad(eta)
        self.create_detector(self._shape, self._pixel_size,
                             construction_mode=self._construction_mode)
        self._two_theta, self._eta, self._distance = float(two_theta), float(eta), float(distance)
        R = self.get_rotation_detector(self._two_theta, self._eta)
        self._direction = R @ np.array([1.0, 0.0, 0.0], dtype=np.float32)
        self._center = self._distance * np.array(
            [np.cos(self._two_theta), np.sin(self._two_theta) * np.sin(self._eta),
             np.sin(self._two_theta) * np.cos(self._eta)], dtype=np.float32)
        c = R @ self._pixel_coordinates + self._center[:, None]
        if self._construction_mode == "shell":
            c = c / np.linalg.norm(c, axis=0, keepdims=True) * self._distance
        self._pixel_coordinates = c

    def position_detector_relative(self, distance, two_theta, eta, degrees=True):
        """Move by increments; reuses the absolute setter (Detector.py:593-618)."""
        dtt = np.deg2rad(two_theta) if degrees else float(two_theta)
        det = np.deg2rad(eta) if degrees else float(eta)
        self.position_detector_absolute(float(self._distance) + float(distance),
                                        float(self._two_theta) + dtt, float(self._eta) + det,
                                        degrees=False)

    def input_pixel_values(self, pixel_values):
        self._pixel_values = pixel_values
        self._pixel_intensity = None

    @property
    def shape(self):
        return self._shape

    @property
    def pixel_size(self):
        return self._pixel_size

    @property
    def pixel_coordinates(self):
        return self._pixel_coordinates

    @property
    def pixel_values(self):
        return self._pixel_values

    @property
    def pixel_intensity(self):
        if self._pixel_intensity is None and self._pixel_values is not None:
            self._pixel_intensity = np.abs(self._pixel_values) ** 2
        return self._pixel_intensity

    @property
    def center(self):
        return self._center

    @property
    def distance(self):
        return self._distance

    @property
    def two_theta(self):
        return self._two_theta

    @property
    def eta(self):
        return self._eta


class Stage:
    """Goniometer motor stack. ``rotation`` maps sample to lab coordinates,
    pos_lab = R @ pos_sample; motors compose in list order, each new rotation
    applied on the left, and a motor's axis is first carried by the motors in
    its coupling list (Stage.py:74-126, 320-382)."""

    DEFAULT_NAMES = ["mu", "phi", "chi", "omega", "x", "y", "z"]
    DEFAULT_TYPES = ["R", "R", "R", "R", "T", "T", "T"]
    DEFAULT_COUPLING = [[None], [0], [0], [0, 1, 2], [0, 1, 2, 3], [0, 1, 2, 3], [0, 1, 2, 3]]
    DEFAULT_AXES = [[0.0, -1.0, 0.0], [0.0, -1.0, 0.0], [-1.0, 0.0, 0.0], [0.0, 0.0, -1.0],
                    [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]]

    def __init__(self):
        self.create_stage()

    def create_stage(self, motor_name=None, motor_type=None, motor_coupling=None,
                     motor_axis=None, motor_value=None):
        self._motor_name = list(motor_name or self.DEFAULT_NAMES)
        self._motor_type = np.array(motor_type or self.DEFAULT_TYPES)
        self._motor_coupling = motor_coupling or self.DEFAULT_COUPLING
        self._motor_axis = np.array(motor_axis or self.DEFAULT_AXES, dtype=np.float64)
        n = len(self._motor_name)
        self._motor_value = np.array(motor_value if motor_value is not None else [0.0] * n,
                                     dtype=np.float64)
        if not (len(self._motor_type) == len(self._motor_coupling) == len(self._motor_axis)
                == self._motor_value.size == n):
            raise ValueError(f"Motor lists must all have {n} entries (one per motor_name).")
        self._rotation = np.eye(3, dtype=np.float32)
        self._translation = np.zeros(3, dtype=np.float32)
        self.get_rotation()
        self.get_translation()

    def motor_index(self, name):
        if name not in self._motor_name:
            raise ValueError(f"Unknown stage motor '{name}'. Stage motors: {self._motor_name}")
        return self._motor_name.index(name)

    get_motor_index = motor_index

    def set_single_motor_value_relative(self, name, value, degrees=True):
        """Add ``value`` to one motor (degrees for rotations when ``degrees``)."""
        i = self.motor_index(name)
        v = float(value)
        if self._motor_type[i] == "R" and degrees:
            v = np.deg2rad(v)
        self._motor_value[i] += v
        self.get_rotation()
        self.get_translation()

    def set_single_motor_value_absolute(self, name, value, degrees=True):
        self.set_motor_value(name, value, degrees)

    @property
    def motor_value(self):
        return self._motor_value

    @property
    def motor_names(self):
        return list(self._motor_name)

    @property
    def motor_types(self):
        return [str(t) for t in self._motor_type]

    def set_motor_value(self, name, value, degrees=True):
        i = self.motor_index(name)
        v = float(value)
        if degrees and self._motor_type[i] == "R":
            v = np.deg2rad(v)
        self._motor_value[i] = v
        self.get_rotation()
        self.get_translation()

    def get_motor_axis(self, idx):
        axes = self._motor_axis.copy()
        for coupled in self._motor_coupling[idx]:
            if coupled is None:
                break
            axes[idx] = axis_rotation(self.get_motor_axis(coupled), self._motor_value[coupled],
                                      dtype=np.float32) @ axes[idx]
        return axes[idx]

    def get_rotation(self):
        R = np.eye(3, dtype=np.float32)
        for i in np.where(self._motor_type == "R")[0]:
            R = axis_rotation(self.get_motor_axis(i), self._motor_value[i], dtype=np.float32) @ R
        self._rotation = R
        return R

    def get_translation(self):
        t = np.zeros(3, dtype=np.float32)
        for i in np.where(self._motor_type == "T")[0]:
            t += self.get_motor_axis(i) * self._motor_value[i]
        self._translation = t
        return t

    @property
    def rotation(self):
        return self._rotation

    @property
    def translation(self):
        return self._translation


class StaticStage:
    """A fixed (rotation, translation) pair with the stage duck type."""

    def __init__(self, rotation=None, translation=None):
        self.rotation = np.asarray(np.eye(3) if rotation is None else rotation, dtype=np.float32)
        self.translation = np.asarray(np.zeros(3) if translation is None else translation,
                                      dtype=np.float32)
