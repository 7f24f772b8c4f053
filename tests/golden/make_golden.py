"""Generate the golden fixtures in tests/golden/ by RUNNING THE REFERENCE.

Run in a container where the reference MOSAIC checkout is importable:

    python tests/golden/make_golden.py /path/to/MOSAIC [--only-depth]

The reference imports pandas for two helpers only; pandas is not installed
here, so ``_shim/pandas.py`` supplies ``unique``/``factorize``/``DataFrame``
with the same results for 1-D label arrays. Everything else runs the
reference's own code: its cffi C kernel ``compute_scattering_cffi``
(Beam.py:621-845), its NumPy twin ``_cpu_scatter_numpy`` (Beam.py:847-953),
``interact_beam_cpu`` (Beam.py:5773-5956), the DABAX parsers
(Beam.py:503-615), ``_ein_bilinear_cpu`` (Beam.py:956-1045), the polarization
state (Beam.py:31-47, 117-149), detector placement (Detector.py:73-741), stage
rotations (Stage.py:252-382), the Gaussian thermal draw (Sample.py:2084-2156,
2321-2334), the free-space propagator (Beam.py:4622-4900, 7945-8022) and the
depth-dependent incident field (Beam.py:956-1045, 5583-5618, 7118-7283).

The fixtures are small .npz files; the GPU machine never needs the reference.
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_dir: str) -> None:
    sys.path[:0] = [os.path.join(HERE, "_shim"), ref_dir]
    import Beam  # noqa: E402
    import Detector  # noqa: E402
    import Sample  # noqa: E402
    import Stage  # noqa: E402

    tmp = tempfile.mkdtemp(prefix="mosaic_golden_")
    B = Beam.beam(directory=os.path.join(tmp, "beam"))
    rng = np.random.default_rng(20261203)
    out = {}

    # ---------------------------------------------------------------- tables
    f0_all = B.parse_f0_db_all("f0_WaasKirf.dat")
    f1f2_all = B.parse_f1f2_db_all("f1f2_CromerLiberman.dat")
    f0z_all = B._build_f0_zero_dict(f0_all)
    elements = ["Cu", "Na", "Cl", "Si", "Fe", "Au", "O", "C"]
    energies = [5000.0, 8000.0, 8979.0, 10000.0, 12000.0, 30000.0, 80000.0]
    out["tab_elements"] = np.array(elements)
    out["tab_energies"] = np.array(energies)
    out["tab_f0"] = np.stack([f0_all[e] for e in elements]).astype(np.float32)
    out["tab_f0z"] = np.array([f0z_all[e] for e in elements])
    out["tab_anom"] = np.array([[complex(B.get_f1f2_from_params(E, f1f2_all[e]))
                                 for E in energies] for e in elements])
    np.savez_compressed(os.path.join(HERE, "tables.npz"), **out)

    # ---------------------------------------------------------- polarization
    pol_cases = [(1.0, None, None), (0.0, None, None), (0.5, None, None), (0.8, None, None),
                 (0.3, None, None), (0.5, (0.0, 0.6, 0.8), 0.7), (0.5, (1.0, 1.0, 0.0), None),
                 (0.9, (1.0, 0.0, 0.0), 0.4)]
    pol_out = []
    for rho, vec, deg in pol_cases:
        B._set_polarization(rho, vec, deg)
        B._direction = np.array([1.0, 0.0, 0.0])
        pol_out.append(B._polarization_state())
    np.savez_compressed(os.path.join(HERE, "polarization.npz"),
                        rho=np.array([c[0] for c in pol_cases]),
                        vec=np.array([c[1] if c[1] is not None else (np.nan,) * 3 for c in pol_cases]),
                        deg=np.array([c[2] if c[2] is not None else np.nan for c in pol_cases]),
                        state=np.array(pol_out))

    # -------------------------------------------------------------- geometry
    det_cases = [((12, 9), (5.5e5, 5.5e5), 2.0e9, 30.0, 20.0),
                 ((16, 16), (5.5e5, 5.5e5), 1.0e10, 34.56, 0.0),
                 ((7, 11), (1.72e6, 1.0e6), 5.0e9, 12.7, -35.0),
                 ((9, 8), (5.5e5, 5.5e5), 1.0e9, 0.0, 0.0)]
    det_out = {}
    for i, (shape, pix, dist, tth, eta) in enumerate(det_cases):
        D = Detector.detector(directory=os.path.join(tmp, f"det{i}"))
        D.create_detector(shape, pix)
        D.position_detector_absolute(dist, tth, eta, degrees=True)
        det_out[f"coords{i}"] = np.asarray(D.pixel_coordinates)
        det_out[f"case{i}"] = np.array([shape[0], shape[1], pix[0], pix[1], dist, tth, eta])
    det_out["n"] = np.array(len(det_cases))
    np.savez_compressed(os.path.join(HERE, "detector.npz"), **det_out)

    stage_vals = [[0.0] * 7, [12.7, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0],
                  [3.0, -20.0, 5.0, 40.0, 1.0, -2.0, 0.5], [0.4, 0.1, -0.3, 0.0, 0.0, 0.0, 0.0]]
    st_rot, st_tr = [], []
    for i, mv in enumerate(stage_vals):
        S = Stage.stage(directory=os.path.join(tmp, f"st{i}"))
        S.create_stage(motor_value=list(np.deg2rad(mv[:4])) + list(mv[4:]))
        st_rot.append(np.asarray(S.get_rotation(), dtype=np.float32))
        st_tr.append(np.asarray(S.get_translation(), dtype=np.float32))
    np.savez_compressed(os.path.join(HERE, "stage.npz"), motor_deg=np.array(stage_vals),
                        rotation=np.array(st_rot), translation=np.array(st_tr))

    # --------------------------------------------------------------- thermal
    pos = (rng.random((1000, 3)) * 40.0 - 20.0).astype(np.float32)
    sam = Sample.sample.__new__(Sample.sample)
    disp = {}
    for sigma, clip, seed, chunk in [(0.08, 1.0, 40, 1), (0.25, 0.3, 7, 3), (0.1, 0.0, 40, 2)]:
        disp[f"{sigma}_{clip}_{seed}_{chunk}"] = Sample.sample.apply_temperature(
            sam, pos.copy(), "gaussian", sigma, clip, seed, chunk)
    np.savez_compressed(os.path.join(HERE, "thermal.npz"), pos=pos,
                        keys=np.array(list(disp.keys())),
                        out=np.stack(list(disp.values())))

    # ------------------------------------------------------------------- Ein
    B.create_beam(10000.0, beam_size=(120.0, 80.0), beam_samples=(33, 21),
                  beam_profile="gaussian", gaussian_waist=(40.0, 30.0))
    wf = (rng.standard_normal((33, 21)) + 1j * rng.standard_normal((33, 21))).astype(np.complex64)
    B.set_wavefield(wf)
    epos = (rng.random((2000, 3)) * 160.0 - 80.0).astype(np.float32)
    z = np.zeros((33, 21), np.float32)
    ein = B._ein_bilinear_cpu(epos, z, z, B._beam_E0_map, B._beam_e1, B._beam_e2,
                              np.array([1, 0, 0], np.float32), B._beam_du, B._beam_dv,
                              B._beam_uc, B._beam_vc, 0.0, 1.0)
    np.savez_compressed(os.path.join(HERE, "ein.npz"), pos=epos, E0=B._beam_E0_map,
                        grid=np.array([B._beam_du, B._beam_dv, B._beam_uc, B._beam_vc]),
                        ein=ein)

    # ---------------------------------------------------- raw kernel (cffi)
    ffi, C = B.compile_compute_scattering_cffi()
    kcases = {}
    det_geo = [(12, 9, 2.0e9, 30.0, 20.0), (10, 10, 3.0e9, 0.4, 0.0), (6, 13, 5.0e8, 60.0, 45.0)]
    flag_sets = [(0, 0, 0, (1.0, None, None)), (1, 1, 1, (1.0, None, None)),
                 (0, 1, 0, (0.3, None, None)), (1, 0, 1, (0.5, None, None)),
                 (0, 1, 1, (0.5, (0.0, 0.6, 0.8), 0.7)), (1, 1, 0, (0.5, None, None))]
    ci = 0
    for gi, (ny, nz, dist, tth, eta) in enumerate(det_geo):
        D = Detector.detector(directory=os.path.join(tmp, f"kd{gi}"))
        D.create_detector((ny, nz), (5.5e5, 5.5e5))
        D.position_detector_absolute(dist, tth, eta, degrees=True)
        cxyz = np.asarray(D.pixel_coordinates).astype(np.float64) / 1e10
        for rf, ap, dc, (rho, vec, deg) in flag_sets:
            n = int(rng.integers(150, 400))
            els = rng.choice(["Cu", "Na", "Cl"], size=n)
            posA = (rng.random((n, 3)) * 60.0 - 30.0).astype(np.float32)
            pos_m = posA.astype(np.float64) / 1e10
            wk = np.stack([f0_all[e] for e in els]).astype(np.float32)
            f0z = np.array([f0z_all[e] for e in els], np.float32)
            an = np.array([B.get_f1f2_from_params(10000.0, f1f2_all[e]) for e in els])
            ar, ai = an.real.astype(np.float32), an.imag.astype(np.float32)
            amp = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
            amp[rng.random(n) < 0.1] = 0
            B._set_polarization(rho, vec, deg)
            B._direction = np.array([1.0, 0.0, 0.0])
            pdeg, ex, ey, ez = B._polarization_state()
            k = 2.0 * np.pi / B._wavelength
            outs = []
            for fn in ("cffi", "numpy"):
                o_r = np.zeros(ny * nz, np.float32)
                o_i = np.zeros(ny * nz, np.float32)
                apr = np.ascontiguousarray(amp.real, dtype=np.float32)
                api = np.ascontiguousarray(amp.imag, dtype=np.float32)
                if fn == "cffi":
                    P = lambda a, t: ffi.cast(t, a.ctypes.data)
                    cc = [np.ascontiguousarray(cxyz[i]) for i in range(3)]
                    pm = np.ascontiguousarray(pos_m)
                    rc = C.compute_scattering_cffi(
                        n, P(pm, "const double *"), P(wk, "const float *"),
                        P(f0z, "const float *"), rf, P(ar, "const float *"),
                        P(ai, "const float *"), P(apr, "const float *"), P(api, "const float *"),
                        ny, nz, P(cc[0], "const double *"), P(cc[1], "const double *"),
                        P(cc[2], "const double *"), float(k), ap, pdeg, ex, ey, ez, dc,
                        P(o_r, "float *"), P(o_i, "float *"))
                    assert rc == 0
                else:
                    B._cpu_scatter_numpy(pos_m, wk, f0z, ar, ai, apr, api, cxyz[0], cxyz[1],
                                         cxyz[2], float(k), bool(rf), ny, nz, bool(ap), pdeg,
                                         (ex, ey, ez), bool(dc), o_r, o_i)
                outs.append(o_r + 1j * o_i)
            pre = f"c{ci}_"
            kcases.update({pre + "pos_m": pos_m, pre + "wk": wk, pre + "f0z": f0z,
                           pre + "anom": ar + 1j * ai, pre + "amp": amp, pre + "cxyz": cxyz,
                           pre + "meta": np.array([ny, nz, rf, ap, dc, k, pdeg, ex, ey, ez]),
                           pre + "out_cffi": outs[0], pre + "out_numpy": outs[1]})
            ci += 1
    kcases["n"] = np.array(ci)
    np.savez_compressed(os.path.join(HERE, "kernel_cases.npz"), **kcases)

    # ------------------------------------------- interact_beam_cpu end to end
    class DuckSample:
        def __init__(self, chunks):
            self._c = chunks
            self.chunk_total = len(chunks)
            self.directory = tmp

        def chunk_atom_count(self, cid):
            return int(self._c[cid - 1][0].shape[0])

        def load_chunk_positions(self, cid, use_gpu=False, raw=False):
            return self._c[cid - 1][0].copy()

        def load_chunk_species(self, cid, use_gpu=False, codes=False):
            return self._c[cid - 1][1].copy()

    chunks = []
    for nA in (1500, 900):
        posA = (rng.random((nA, 3)) * 50.0 - 25.0).astype(np.float32)
        chunks.append((posA, rng.choice(np.array(["Na", "Cl", "Cu"]), size=nA)))
    duck = DuckSample(chunks)
    D = Detector.detector(directory=os.path.join(tmp, "e2e_det"))
    D.create_detector((14, 10), (5.5e5, 5.5e5))
    D.position_detector_absolute(1.0e9, 25.0, 10.0, degrees=True)
    S = Stage.stage(directory=os.path.join(tmp, "e2e_st"))
    S.create_stage(motor_value=list(np.deg2rad([4.0, 10.0, -3.0, 20.0])) + [1.0, 0.5, -0.5])
    S.get_rotation(); S.get_translation()
    B.create_beam(12000.0, beam_size=(70.0, 60.0), beam_samples=(64, 48),
                  beam_profile="gaussian", gaussian_waist=(30.0, 25.0), pol_perp_rate=0.9)
    e2e = {}
    for i, (rf, ap, dc) in enumerate([(0, 1, 0), (1, 1, 1), (0, 0, 1)]):
        e2e[f"out{i}"] = B.interact_beam_cpu(duck, D.pixel_coordinates, D.shape, S, None,
                                             remove_forward_component=bool(rf),
                                             apply_polarization=bool(ap),
                                             apply_spherical_decay=bool(dc))
        e2e[f"flags{i}"] = np.array([rf, ap, dc])
    e2e.update(pos0=chunks[0][0], spc0=chunks[0][1], pos1=chunks[1][0], spc1=chunks[1][1],
               coords=np.asarray(D.pixel_coordinates), shape=np.array(D.shape),
               rotation=S.rotation, translation=S.translation, energy=np.array(12000.0),
               E0=B._beam_E0_map, grid=np.array([B._beam_du, B._beam_dv, B._beam_uc, B._beam_vc]),
               pol=np.array(B._polarization_state()), wavelength=np.array(B._wavelength))
    np.savez_compressed(os.path.join(HERE, "interact_cpu.npz"), **e2e)

    # ------------------------------------------------------------ propagation
    pffi, plib = B.compile_propagation_multiplier_cffi()
    Fs = (rng.standard_normal((16, 24)) + 1j * rng.standard_normal((16, 24))).astype(np.complex64)
    prop = {}
    for i, (d, zz) in enumerate([(5.5e-6, 0.01), (2.0e-11, 3e-9), (1.0e-6, -0.002)]):
        ky = ((2.0 * np.pi) * np.fft.fftfreq(24, d=d)).astype(np.float32)
        kz = ((2.0 * np.pi) * np.fft.fftfreq(16, d=d)).astype(np.float32)
        G = Fs.copy()
        kk = np.float32(2.0 * np.pi / B._wavelength)
        plib.prop_mul_cpu(np.int32(24), np.int32(16), pffi.cast("const float*", ky.ctypes.data),
                          pffi.cast("const float*", kz.ctypes.data), kk, np.float32(zz),
                          pffi.cast("float*", G.ctypes.data))
        prop[f"mul{i}"] = G
        prop[f"mulcase{i}"] = np.array([d, zz])
        prop[f"ky{i}"] = ky
        prop[f"kz{i}"] = kz
    field = (rng.standard_normal((20, 28)) + 1j * rng.standard_normal((20, 28))).astype(np.complex64)
    prop["field"] = field
    prop["k"] = np.array(np.float32(2.0 * np.pi / B._wavelength))
    prop["Fs"] = Fs
    prop["wavelength"] = np.array(B._wavelength)
    for i, (dy, zz) in enumerate([(1e-6, 0.003), (5.5e-5, 0.5)]):
        prop[f"asp{i}"] = B._angular_spectrum_propagate_cpu(field, dy, dy, zz, plib, pffi)
        prop[f"aspcase{i}"] = np.array([dy, zz])
    np.savez_compressed(os.path.join(HERE, "propagation.npz"), **prop)
    depth_ein(B)
    print("golden fixtures written to", HERE)


class _Sample:
    """Minimal chunk duck type for the reference's depth-Ein helpers."""

    def __init__(self, chunks):
        self.chunks = chunks
        self.chunk_total = len(chunks)

    def load_chunk_positions(self, cid, use_gpu=False, raw=False):
        return self.chunks[cid - 1][0].copy()

    def load_chunk_species(self, cid, use_gpu=False, codes=False):
        return self.chunks[cid - 1][1].copy()


class _Stage:
    def __init__(self, R, T):
        self.rotation = R
        self.translation = T


def depth_ein(B):
    """Depth-dependent incident field: the reference's transmission map
    (_compute_beam_column_A_map_cpu, Beam.py:7118-7283), depth window
    (_compute_global_depth_bounds, Beam.py:5583-5618) and per-atom Ein
    (_ein_bilinear_cpu, Beam.py:956-1045) on a small gold/iron slab."""
    rng = np.random.default_rng(4963)
    a = 4.078
    cells = np.stack(np.meshgrid(np.arange(30), np.arange(10), np.arange(10), indexing="ij"), -1)
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    pos = ((cells.reshape(-1, 1, 3) + basis[None]) * a).reshape(-1, 3)
    pos = (pos - pos.mean(0)).astype(np.float32)
    spc = np.where(rng.random(pos.shape[0]) < 0.8, "Au", "Fe")
    half = pos.shape[0] // 2
    sample = _Sample([(pos[:half], spc[:half]), (pos[half:], spc[half:])])
    c, s_ = np.cos(np.radians(3.0)), np.sin(np.radians(3.0))
    R = np.array([[c, -s_, 0], [s_, c, 0], [0, 0, 1]], np.float32)
    T = np.array([1.5, -2.0, 0.5], np.float32)
    stage = _Stage(R, T)
    B.create_beam(10000.0, beam_size=(60.0, 60.0), beam_samples=(61, 61))
    A = B._compute_beam_column_A_map_cpu(sample, stage)
    s_min, s_max = B._compute_global_depth_bounds(sample, stage)
    tau = (-np.log(np.abs(A) + np.float32(1e-20))).astype(np.float32)
    phi = np.angle(A).astype(np.float32)
    lab = (pos @ R.T + T).astype(np.float32)
    ein = B._ein_bilinear_cpu(lab, tau, phi, B._beam_E0_map.astype(np.complex64),
                              B._beam_e1.astype(np.float32), B._beam_e2.astype(np.float32),
                              np.array([1, 0, 0], np.float32), B._beam_du, B._beam_dv,
                              B._beam_uc, B._beam_vc, s_min, s_max)
    np.savez_compressed(os.path.join(HERE, "depth_ein.npz"), pos=pos, spc=spc, R=R, T=T,
                        grid=np.array([B._beam_du, B._beam_dv, B._beam_uc, B._beam_vc]),
                        E0=B._beam_E0_map, A=A, s=np.array([s_min, s_max]), ein=ein,
                        wavelength=np.array(B._wavelength), energy=np.array(B._energy))


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout> [--only-depth]")
    ref = sys.argv[1]
    if len(sys.argv) > 2 and sys.argv[2] == "--only-depth":
        sys.path[:0] = [os.path.join(HERE, "_shim"), ref]
        import Beam  # noqa: E402
        depth_ein(Beam.beam(directory=tempfile.mkdtemp(prefix="mosaic_golden_")))
    else:
        main(ref)
