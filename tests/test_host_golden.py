"""Host-side logic of the package against the reference's own outputs:
tables, detector and stage geometry, polarization, thermal displacement and
the beam grid must be bit-identical (they feed the kernels unchanged)."""
import numpy as np
import pytest

from mosaic_gb300 import ChunkedSample, Detector, Stage, polarization_state, thermal_displacement
from mosaic_gb300.beam import beam as Beam
from mosaic_gb300.tables import ScatteringTables, f0_at_zero, parse_f0_file


def test_tables_bit_identical(golden):
    t = golden("tables.npz")
    T = ScatteringTables()
    for i, el in enumerate(t["tab_elements"]):
        el = str(el)
        assert np.array_equal(T.row(el), t["tab_f0"][i])
        assert T.f0_zero(el) == t["tab_f0z"][i]
        for j, E in enumerate(t["tab_energies"]):
            assert T.anomalous(el, float(E)) == t["tab_anom"][i, j]


def test_table_parser_format(tmp_path):
    f = tmp_path / "f0.dat"
    f.write_text("#F x\n#S 29 Cu\n#N 11\n 1 2 3 4 5 6 7 8 9 10 11\n#S 8 O\n1 2 3\n"
                 " 0.5 0 0 0 0 1 1 1 1 1 1\n")
    rows = parse_f0_file(str(f))
    assert set(rows) == {"Cu", "O"}
    assert rows["Cu"].dtype == np.float32 and rows["Cu"][5] == 6
    assert f0_at_zero(rows["O"]) == 1.5


def test_bundled_table_missing_element_is_loud():
    T = ScatteringTables()
    assert T.has("Cu1+")
    with pytest.raises(KeyError):
        T.anomalous("Cu1+", 10000.0)


def test_detector_geometry_bit_identical(golden):
    d = golden("detector.npz")
    for i in range(int(d["n"])):
        ny, nz, py, pz, dist, tth, eta = d[f"case{i}"]
        D = Detector()
        D.create_detector((int(ny), int(nz)), (py, pz))
        D.position_detector_absolute(dist, tth, eta)
        assert D.pixel_coordinates.dtype == d[f"coords{i}"].dtype
        assert np.array_equal(D.pixel_coordinates, d[f"coords{i}"]), i


def test_stage_rotation_bit_identical(golden):
    s = golden("stage.npz")
    for i, mv in enumerate(s["motor_deg"]):
        S = Stage()
        S.create_stage(motor_value=list(np.deg2rad(mv[:4])) + list(mv[4:]))
        assert S.rotation.dtype == np.float32
        assert np.array_equal(S.rotation, s["rotation"][i])
        assert np.array_equal(S.translation, s["translation"][i])


def test_polarization_state(golden):
    p = golden("polarization.npz")
    for i in range(len(p["rho"])):
        vec = None if np.isnan(p["vec"][i][0]) else p["vec"][i]
        deg = None if np.isnan(p["deg"][i]) else float(p["deg"][i])
        assert np.array_equal(np.array(polarization_state(p["rho"][i], vec, deg)), p["state"][i])


def test_thermal_displacement_bit_identical(golden):
    t = golden("thermal.npz")
    for key, ref in zip(t["keys"], t["out"]):
        sigma, clip, seed, chunk = str(key).split("_")
        got = thermal_displacement(t["pos"], float(sigma), float(clip), int(seed), int(chunk))
        assert got.dtype == np.float32
        assert np.array_equal(got, ref), key


def test_chunked_sample_api():
    pos = np.arange(12, dtype=np.float32).reshape(4, 3)
    s = ChunkedSample([(pos, np.array(["Cu", "O", "Cu", "Cu"])), (pos[:1], np.array(["O"]))],
                      thermal=dict(sigma=0.1, max_displacement=1.0, seed=40))
    assert s.chunk_total == 2 and s.chunk_atom_count(1) == 4 and s.chunk_atom_count(2) == 1
    codes, labels = s.load_chunk_species(1, codes=True)
    assert list(labels[codes]) == ["Cu", "O", "Cu", "Cu"]
    assert np.array_equal(s.load_chunk_positions(1, raw=True), pos)
    assert np.array_equal(s.load_chunk_positions(1), thermal_displacement(pos, 0.1, 1.0, 40, 1))
    assert not np.array_equal(s.load_chunk_positions(1), s.load_chunk_positions(2)[:1].repeat(4, 0))


def test_beam_grid_and_wavefield(golden):
    e = golden("interact_cpu.npz")
    B = Beam()
    B.create_beam(12000.0, beam_size=(70.0, 60.0), beam_samples=(64, 48),
                  beam_profile="gaussian", gaussian_waist=(30.0, 25.0), pol_perp_rate=0.9)
    # exact on the machine that made the fixture; np.exp's last bit may differ elsewhere
    assert np.allclose(B._beam_E0_map, e["E0"], rtol=1e-6, atol=0)
    assert np.array_equal(np.array(B._beam_grid()), e["grid"])
    assert np.array_equal(np.array(B._polarization_state()), e["pol"])
    assert B._wavelength == float(e["wavelength"])
    with pytest.raises(ValueError):
        B.set_wavefield(np.zeros((3, 3)))
    with pytest.raises(ValueError):
        B.set_wavefield(np.full((64, 48), np.nan))


def test_forward_beam_required_and_no_cpu_path():
    B = Beam()
    B.create_beam(10000.0)
    with pytest.raises(ValueError):
        B._require_forward_beam((1.0, 0.5, 0.0))
    with pytest.raises(RuntimeError):
        B.atomic_scattering_kinematic(ChunkedSample([]), Detector(), None, use_gpu=False)


def test_phase_tolerance_semantics():
    B = Beam()
    B.set_phase_tolerance(-1)
    assert B._phase_tol_rad == 1e-3
    B.set_phase_tolerance("x")
    assert B._phase_tol_rad == 1e-3
    B.set_phase_tolerance(2e-4)
    assert B._phase_tol_rad == 2e-4
