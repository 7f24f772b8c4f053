"""Pin the CPU oracle to the reference: every fixture here was produced by
running the reference itself (tests/golden/make_golden.py)."""
import numpy as np

import oracle


def test_oracle_kernel_matches_reference_kernels(golden):
    d = golden("kernel_cases.npz")
    assert int(d["n"]) >= 18
    for i in range(int(d["n"])):
        p = f"c{i}_"
        ny, nz, rf, ap, dc, k, pdeg, ex, ey, ez = d[p + "meta"]
        a, amp, c = d[p + "anom"], d[p + "amp"], d[p + "cxyz"]
        got = oracle.scatter_f64(d[p + "pos_m"], d[p + "wk"], d[p + "f0z"], a.real, a.imag,
                                 amp.real, amp.imag, c[0], c[1], c[2], k, int(ny), int(nz), rf, ap,
                                 (pdeg, ex, ey, ez), dc, n_threads=3)
        m = np.abs(got).max()
        # NumPy twin: same uncontracted double arithmetic, output rounded to float32.
        assert np.abs(got - d[p + "out_numpy"]).max() / m <= 2e-7, i
        # cffi kernel: built -O3 -march=native, which contracts FMAs and moves the
        # ~1e10 rad absolute phase by ~1e-6 rad.
        assert np.abs(got - d[p + "out_cffi"]).max() / m <= 1e-5, i


def test_oracle_threads_do_not_change_result(golden):
    d = golden("kernel_cases.npz")
    p = "c1_"
    ny, nz, rf, ap, dc, k, pdeg, ex, ey, ez = d[p + "meta"]
    a, amp, c = d[p + "anom"], d[p + "amp"], d[p + "cxyz"]
    args = (d[p + "pos_m"], d[p + "wk"], d[p + "f0z"], a.real, a.imag, amp.real, amp.imag,
            c[0], c[1], c[2], k, int(ny), int(nz), rf, ap, (pdeg, ex, ey, ez), dc)
    r1 = oracle.scatter_f64(*args, n_threads=1)
    r4 = oracle.scatter_f64(*args, n_threads=4)
    assert np.abs(r1 - r4).max() <= 1e-14 * np.abs(r1).max()


def test_oracle_interact_matches_reference_interact_beam_cpu(golden):
    e = golden("interact_cpu.npz")
    t = golden("tables.npz")
    from mosaic_gb300.tables import ScatteringTables
    T = ScatteringTables()
    chunks = [(e["pos0"], e["spc0"]), (e["pos1"], e["spc1"])]
    labels = ["Na", "Cl", "Cu"]
    for i in range(3):
        rf, ap, dc = (bool(v) for v in e[f"flags{i}"])
        got = oracle.interact_cpu(chunks, e["coords"], tuple(e["shape"]), e["rotation"],
                                  e["translation"], float(e["energy"]), T.f0,
                                  {l: T.f0_zero(l) for l in labels}, T.f1f2, e["E0"], e["grid"],
                                  tuple(e["pol"]), remove_forward=rf, apply_polarization=ap,
                                  spherical_decay=dc)
        ref = e[f"out{i}"]
        assert got.shape == ref.shape
        assert np.abs(got - ref).max() / np.abs(ref).max() <= 1e-5, i
    assert t["tab_f0"].shape[1] == 11


def test_oracle_ein_bilinear_bit_exact(golden):
    d = golden("ein.npz")
    du, dv, uc, vc = d["grid"]
    got = oracle.ein_bilinear(d["pos"], d["E0"], du, dv, uc, vc)
    assert np.array_equal(got, d["ein"])
    assert np.any(got == 0) and np.any(got != 0)   # some atoms fall outside the grid


def test_oracle_polarization_and_anomalous(golden):
    p = golden("polarization.npz")
    for i in range(len(p["rho"])):
        vec = None if np.isnan(p["vec"][i][0]) else p["vec"][i]
        deg = None if np.isnan(p["deg"][i]) else float(p["deg"][i])
        assert np.array_equal(np.array(oracle.polarization_state(p["rho"][i], vec, deg)),
                              p["state"][i])
    t = golden("tables.npz")
    from mosaic_gb300.tables import ScatteringTables
    T = ScatteringTables()
    for i, el in enumerate(t["tab_elements"]):
        for j, E in enumerate(t["tab_energies"]):
            assert oracle.anomalous(float(E), T.f1f2[str(el)]) == t["tab_anom"][i, j]


def test_oracle_prop_mul_matches_reference(golden):
    d = golden("propagation.npz")
    k = float(d["k"])
    for i in range(3):
        dd, z = d[f"mulcase{i}"]
        got = oracle.prop_mul_f64(d["Fs"], d[f"ky{i}"], d[f"kz{i}"], k, z)
        ref = d[f"mul{i}"]
        # the reference evaluates the phase in float32 (cosf/sinf)
        scale = np.abs(d["Fs"]).max()
        assert np.abs(got - ref).max() / scale <= 5e-5, i


def test_depth_ein_oracle_matches_reference(golden):
    """Transmission map, depth window and depth-dependent Ein of a gold/iron
    slab, against the reference's own outputs (Beam.py:956-1045, 5583-5618,
    7118-7283)."""
    d = golden("depth_ein.npz")
    t = golden("tables.npz")
    els = list(t["tab_elements"])
    e_idx = list(t["tab_energies"]).index(float(d["energy"]))
    spc = d["spc"].astype(str)
    fr = np.zeros(spc.size, np.float32)
    fi = np.zeros(spc.size, np.float32)
    for el in ("Au", "Fe"):
        m = spc == el
        c = t["tab_anom"][els.index(el), e_idx]
        fr[m] = np.float32(t["tab_f0z"][els.index(el)]) + np.float32(c.real)
        fi[m] = np.float32(c.imag)
    lab = (d["pos"] @ d["R"].T + d["T"]).astype(np.float32)
    du, dv, uc, vc = d["grid"]
    A = oracle.column_map(lab, fr, fi, d["A"].shape, du, dv, uc, vc, float(d["wavelength"]) * 1e10)
    ref = d["A"]
    assert np.allclose(A, ref, rtol=0, atol=2e-6), np.abs(A - ref).max()
    assert np.allclose([lab[:, 0].min(), lab[:, 0].max()], d["s"], rtol=0, atol=1e-5)
    tau = (-np.log(np.abs(ref) + np.float32(1e-20))).astype(np.float32)
    phi = np.angle(ref).astype(np.float32)
    ein = oracle.ein_depth(lab, d["E0"], tau, phi, du, dv, uc, vc, d["s"][0], d["s"][1])
    assert np.allclose(ein, d["ein"], rtol=0, atol=1e-6 * np.abs(d["ein"]).max())


def test_depth_blur_matches_oracle():
    """The host-side Gaussian blur of the depth maps (torch FFT, the map's
    device) against the reference's NumPy form."""
    import torch
    from mosaic_gb300 import engine
    rng = np.random.default_rng(3)
    m = rng.standard_normal((40, 33)).astype(np.float32)
    for rad in (1, 3, 6):
        got = engine._gauss_blur(torch.tensor(m), rad).numpy()
        assert np.allclose(got, oracle.blur_map(m, rad), rtol=0, atol=1e-6), rad


def test_reference_kernel_built_from_its_source(golden):
    """The reference's own compute_scattering_cffi, compiled from its source
    by oracle/ref_build.py (skipped where neither a reference checkout nor
    the extracted source is present), reproduces the fixtures it made, and
    the oracle; it is the CPU baseline the benchmark times."""
    import pytest
    if oracle.ref_lib() is None:
        pytest.skip("reference source not available on this machine")
    d = golden("kernel_cases.npz")
    for i in range(int(d["n"])):
        p = f"c{i}_"
        ny, nz, rf, ap, dc, k, pdeg, ex, ey, ez = d[p + "meta"]
        a, amp, c = d[p + "anom"], d[p + "amp"], d[p + "cxyz"]
        args = (d[p + "pos_m"], d[p + "wk"], d[p + "f0z"], a.real, a.imag, amp.real, amp.imag,
                c[0], c[1], c[2], k, int(ny), int(nz), rf, ap, (pdeg, ex, ey, ez), dc)
        got = oracle.scatter_ref(*args, n_threads=3, slice_atoms=100)
        m = np.abs(got).max()
        # float32 output per slice; contraction as the host compiler chooses
        assert np.abs(got - d[p + "out_numpy"]).max() / m <= 1e-5, i
        assert np.abs(got - d[p + "out_cffi"]).max() / m <= 1e-5, i
        assert np.abs(got - oracle.scatter_f64(*args, n_threads=2)).max() / m <= 1e-5, i
