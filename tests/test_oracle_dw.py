"""The oracle's Debye-Waller branch against its closed form.

The reference has no Debye-Waller factor (thermal motion enters only as
explicit displacements, Sample.py:790-812); this library adds exp(-B s^2),
s = sin(theta)/lambda = Q / (4 pi), per species, default off. These CPU tests
pin the oracle's restatement of it on the cases where the sum has a closed
form, so that the GPU kernels can be held to the oracle.
"""
import numpy as np

import oracle
from mosaic_gb300.tables import ScatteringTables, f0_value

R_E = 2.81794092e-15


def _pixels(n=(7, 5), dist=2e9, tth=30.0):
    from mosaic_gb300 import Detector
    D = Detector()
    D.create_detector(n, (5.5e5, 5.5e5))
    D.position_detector_absolute(dist, tth, 15.0)
    return np.asarray(D.pixel_coordinates, np.float64) / 1e10, D.shape


def test_single_atom_debye_waller_closed_form():
    """One atom at the origin: A = r_e (f0(Q) + f' + i f'') exp(-B s^2) exp(i k r)."""
    T = ScatteringTables()
    E = 9000.0
    k = 2.0 * np.pi / (12398.419843320026 / E * 1e-10)
    c, (ny, nz) = _pixels()
    row = T.row("Fe")
    an = T.anomalous("Fe", E)
    r = np.linalg.norm(c, axis=0)
    Q = k * np.sqrt(2.0 * (1.0 - c[0] / r))
    s2 = (Q * 0.25e-10 / np.pi) ** 2
    f = f0_value(row, s2) + an
    for B in (0.0, 0.35, 1.7, 6.0):
        got = oracle.scatter_f64(np.zeros((1, 3)), row[None], [T.f0_zero("Fe")], [an.real], [an.imag],
                                 [1.0], [0.0], c[0], c[1], c[2], k, ny, nz, dw_b=[B], n_threads=1)
        Bf = float(np.float32(B))   # B is stored as float32, as the kernels take it
        ref = R_E * f * np.exp(-Bf * s2) * np.exp(1j * np.fmod(k * r, 2.0 * np.pi))
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), B
        if B:
            # the factor is visible: at 30 deg it lowers |A| by exp(-B s^2)
            assert np.abs(np.abs(got) / (R_E * np.abs(f)) - np.exp(-Bf * s2)).max() < 1e-12


def test_debye_waller_zero_is_no_factor_and_is_per_species():
    """B = 0 reproduces the sum without the factor bit for bit, and each
    species' B scales only that species' terms (linearity of the sum)."""
    T = ScatteringTables()
    E = 10000.0
    k = 2.0 * np.pi / (12398.419843320026 / E * 1e-10)
    rng = np.random.default_rng(5)
    n = 300
    pos = (rng.random((n, 3)) - 0.5) * 40e-10
    spc = np.where(rng.random(n) < 0.5, "Na", "Cl")
    wk = np.stack([T.row(e) for e in spc])
    f0z = np.array([T.f0_zero(e) for e in spc], np.float32)
    an = np.array([T.anomalous(e, E) for e in spc])
    c, (ny, nz) = _pixels((6, 4))
    args = (pos, wk, f0z, an.real, an.imag, np.ones(n), np.zeros(n), c[0], c[1], c[2], k, ny, nz)
    kw = dict(apply_pol=True, pol=(1.0, 0.0, 1.0, 0.0), n_threads=2)
    plain = oracle.scatter_f64(*args, **kw)
    zero = oracle.scatter_f64(*args, dw_b=np.zeros(n), **kw)
    assert np.array_equal(plain, zero)
    b = np.where(spc == "Na", 1.1, 0.6)
    both = oracle.scatter_f64(*args, dw_b=b, **kw)
    # the sum over Na atoms with B_Na plus the sum over Cl atoms with B_Cl
    parts = 0
    for el, B in (("Na", 1.1), ("Cl", 0.6)):
        m = spc == el
        sub = (pos[m], wk[m], f0z[m], an.real[m], an.imag[m], np.ones(m.sum()), np.zeros(m.sum()),
               c[0], c[1], c[2], k, ny, nz)
        parts = parts + oracle.scatter_f64(*sub, dw_b=np.full(m.sum(), B), **kw)
    assert np.abs(both - parts).max() <= 1e-12 * np.abs(both).max()
    assert np.abs(both - plain).max() > 1e-3 * np.abs(plain).max()
