"""Analytic known answers for both kernels: two-atom fringes, forward
coherence (N atoms on the beam axis scatter in phase into the forward pixel:
|A|^2 = N^2 r_e^2 |f(0)|^2), and the far-field limit of the near-field sum.

The references are computed in double from the relative phase
k (x_a + |P - a| - |P|), which keeps the ~1e10 rad absolute phase out of the
arithmetic."""
import numpy as np
import pytest

from mosaic_gb300 import Detector, StaticStage
from mosaic_gb300.beam import beam as Beam
from mosaic_gb300.sample import ChunkedSample
from mosaic_gb300.tables import f0_value

from helpers import rel_intensity

pytestmark = pytest.mark.gpu
R_E = 2.81794092e-15


def _f(B, el, Q):
    s2 = (Q * 0.25e-10 / np.pi) ** 2
    return f0_value(B.tables.row(el), s2) + B.tables.anomalous(el, B._energy)


def _exact(B, pos_A, el, coords_A, decay=False):
    """Near-field sum with relative phases, f at each atom-pixel Q."""
    a = np.asarray(pos_A, np.float64) / 1e10
    P = np.asarray(coords_A, np.float64).T / 1e10              # (P, 3)
    R0 = np.linalg.norm(P, axis=1)
    out = np.zeros(P.shape[0], complex)
    for j in range(a.shape[0]):
        d = P - a[j]
        r = np.linalg.norm(d, axis=1)
        Q = B.k * np.sqrt(np.maximum(2 * (1 - d[:, 0] / r), 0))
        ph = B.k * (a[j, 0] + (r - R0))
        amp = R_E * _f(B, el, Q) * (R0 / r if decay else 1.0)
        out += amp * np.exp(1j * ph)
    return out


@pytest.mark.parametrize("fast", [False, True])
def test_two_atom_fringes(cuda, fast):
    B = Beam()
    B.create_beam(12000.0, beam_size=(200.0, 200.0))
    B._use_fast_kernel = fast
    pos = np.array([[0.0, -15.0, 0.0], [0.0, 15.0, 0.0]], np.float32)   # 30 A apart along y
    D = Detector()
    D.create_detector((40, 3), (2.0e6, 2.0e6))
    D.position_detector_absolute(1.0e9, 6.0, 0.0)
    got = B.atomic_scattering_kinematic(ChunkedSample([(pos, np.array(["Fe", "Fe"]))]), D,
                                        StaticStage(), return_double=True).reshape(-1)
    ref = _exact(B, pos, "Fe", D.pixel_coordinates)
    I, Ir = np.abs(got) ** 2, np.abs(ref) ** 2
    # several fringes across the detector, visibility ~1
    assert Ir.min() < 0.1 * Ir.max()
    # FP64 plain: the reference formulation's absolute phase k (x + r) ~ 6e9 rad
    # carries ~1e-6 rad of double rounding per term
    assert np.abs(I - Ir).max() <= (1e-4 if fast else 2e-6) * Ir.max()


@pytest.mark.parametrize("fast", [False, True])
def test_forward_coherence_n_squared(cuda, fast):
    B = Beam()
    B.create_beam(10000.0, beam_size=(400.0, 400.0))
    B._use_fast_kernel = fast
    n = 777
    x = np.linspace(-150.0, 150.0, n).astype(np.float32)
    pos = np.stack([x, np.zeros(n, np.float32), np.zeros(n, np.float32)], 1)
    D = Detector()
    D.create_detector((3, 3), (5.5e5, 5.5e5))
    D.position_detector_absolute(5.0e9, 0.0, 0.0)              # centre pixel on the beam axis
    got = B.atomic_scattering_kinematic(ChunkedSample([(pos, np.array(["Cu"] * n))]), D,
                                        StaticStage(), return_double=True)
    centre = got[1, 1]
    f0 = _f(B, "Cu", 0.0)
    assert abs(abs(centre) ** 2 / (n * R_E * abs(f0)) ** 2 - 1.0) <= (1e-4 if fast else 1e-9)


def test_far_field_limit(cuda):
    """A 1,000-atom cluster seen from 10 m: the split kernel against the
    Fraunhofer sum r_e f e^{ik|P|} sum_a e^{ik(x_a - u.a)}, whose neglected
    terms are k a^2 / 2R ~ 1e-8 rad here."""
    rng = np.random.default_rng(2)
    B = Beam()
    B.create_beam(10000.0, beam_size=(300.0, 300.0))
    B._use_fast_kernel = True
    pos = (rng.random((1000, 3)) * 40 - 20).astype(np.float32)
    D = Detector()
    D.create_detector((16, 12), (1.0e6, 1.0e6))
    D.position_detector_absolute(1.0e11, 20.0, 0.0)
    got = B.atomic_scattering_kinematic(ChunkedSample([(pos, np.array(["Ni"] * 1000))]), D,
                                        StaticStage(), return_double=True).reshape(-1)
    assert B.last_run["path"] == "split_f32"
    P = np.asarray(D.pixel_coordinates, np.float64).T / 1e10
    u = P / np.linalg.norm(P, axis=1, keepdims=True)
    a = pos.astype(np.float64) / 1e10
    Q = B.k * np.sqrt(2 * (1 - u[:, 0]))
    ff = R_E * _f(B, "Ni", Q) * np.exp(1j * B.k * (a[:, 0][None, :] - u @ a.T)).sum(1)
    assert rel_intensity(got, ff) <= 1e-4, rel_intensity(got, ff)
