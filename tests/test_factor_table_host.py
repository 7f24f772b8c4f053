"""What the per-(species, pixel) factor table approximates, measured on the
CPU in FP64: the scattering factor (f0 + f' + i f'') sqrt(P_pol) taken at
each pixel's own direction instead of at the direction from each atom to
the pixel, as the reference evaluates it per (atom, pixel)
(Beam.py:770-806). For a sample that the host admits (2 (|o| + r) / R0 below
1e-6) the field changes by far less than the 1e-4 intensity budget, and
the change grows with the excursion as that bound says.
"""
import numpy as np
import pytest

from mosaic_gb300 import engine
from mosaic_gb300.tables import ScatteringTables, f0_value


def _fields(extent_m, dist_m, n_atoms=1500, npix=8):
    rng = np.random.default_rng(4)
    tab = ScatteringTables()
    E = 10000.0
    lam = 12398.419843320026 / E * 1e-10
    k = 2 * np.pi / lam
    a = rng.uniform(-0.5, 0.5, (n_atoms, 3)) * extent_m          # atoms (m)
    two_theta = 2 * np.arcsin(lam / (2 * 2.0871e-10))              # Cu (111)
    centre = dist_m * np.array([np.cos(two_theta), 0.0, np.sin(two_theta)])
    off = (np.arange(npix) - (npix - 1) / 2) * 55e-6
    Y, Z = np.meshgrid(off, off)
    P = centre + np.stack([np.zeros(Y.size), Y.ravel(), Z.ravel()], 1)   # pixels (m)
    row = tab.row("Cu")
    anom = tab.anomalous("Cu", E)
    e_pol = np.array([0.0, 1.0, 0.0])                              # sigma polarised
    sf = k * 0.25e-10 / np.pi

    def factor(u):
        """(f0 + f' + i f'') sqrt(P) at unit directions u (..., 3)."""
        s2 = sf * sf * np.sum((np.array([1.0, 0.0, 0.0]) - u) ** 2, axis=-1)
        er = u @ e_pol
        pol = np.clip(1.0 - er * er, 0.0, 1.0)
        return (f0_value(row, s2) + anom) * np.sqrt(pol)

    d = P[None, :, :] - a[:, None, :]                              # (atoms, pixels, 3)
    r = np.linalg.norm(d, axis=-1)
    phase = k * (a[:, 0:1] + r)
    per_atom = (factor(d / r[..., None]) * np.exp(1j * phase)).sum(0)
    u_pix = P / np.linalg.norm(P, axis=1, keepdims=True)
    per_pixel = factor(u_pix) * np.exp(1j * phase).sum(0)
    return per_atom, per_pixel


@pytest.mark.parametrize("extent_m,dist_m", [(60e-9, 1.0), (60e-9, 0.5), (20e-9, 0.2)])
def test_table_error_far_inside_the_budget(extent_m, dist_m):
    """Admitted geometries (2 (|o| + r) / R0 < 1e-6): the table changes the
    intensity by < 1e-6 of its peak (the budget is 1e-4)."""
    excursion = 2 * (np.sqrt(3) * extent_m / 2) / dist_m
    assert excursion < engine.FACTOR_TABLE_EXCURSION
    exact, table = _fields(extent_m, dist_m)
    I, It = np.abs(exact) ** 2, np.abs(table) ** 2
    err = np.abs(It - I).max() / I.max()
    assert err < 1e-6, err


def test_table_error_grows_with_the_excursion():
    """Ten times the excursion, about ten times the change: the bound's
    scaling (the direction to any atom differs from the pixel's by at most
    the excursion)."""
    errs = []
    for extent in (2e-7, 2e-6):
        exact, table = _fields(extent, 0.1, n_atoms=800)
        errs.append(np.abs(table - exact).max() / np.abs(exact).max())
    assert 4.0 < errs[1] / errs[0] < 25.0, errs
