"""The reference's on-disk sample format (Sample.py:543-676, 735-872) read
directly: atomic_positions_{i}.npy, atomic_species_{i}.npy (codes with the
label table in sample_metadata.json, or labels), thermal draw on load."""
import json
import os

import numpy as np

from mosaic_gb300 import ChunkedSample, DiskSample, write_sample


def _chunks(rng):
    out = []
    for n in (50, 0, 37):
        pos = (rng.random((n, 3)) * 20).astype(np.float32)
        spc = rng.choice(np.array(["Cu", "Ni", "O"]), n)
        out.append((pos, spc))
    return out


def test_round_trip_and_header_counts(tmp_path):
    rng = np.random.default_rng(0)
    ch = _chunks(rng)
    write_sample(tmp_path, ch)
    meta = json.load(open(os.path.join(tmp_path, "sample_metadata.json")))
    assert meta["chunk_total"] == 3
    s = DiskSample(tmp_path)
    assert s.chunk_total == 3 and s.n_atoms == 87
    for i, (pos, spc) in enumerate(ch, start=1):
        assert s.chunk_atom_count(i) == len(pos)
        assert np.array_equal(s.load_chunk_positions(i), pos)
        assert np.array_equal(s.load_chunk_species(i), spc)
        codes, labels = s.load_chunk_species(i, codes=True)
        assert np.array_equal(labels[codes], spc)


def test_thermal_draw_matches_the_in_memory_sample(tmp_path):
    rng = np.random.default_rng(1)
    ch = _chunks(rng)
    write_sample(tmp_path, ch)
    th = dict(sigma=0.08, max_displacement=1.0, seed=40)
    a, b = DiskSample(tmp_path, thermal=th), ChunkedSample(ch, thermal=th)
    for i in range(1, 4):
        assert np.array_equal(a.load_chunk_positions(i), b.load_chunk_positions(i))
        assert np.array_equal(a.load_chunk_positions(i, raw=True), ch[i - 1][0])


def test_label_files_and_bad_codes(tmp_path):
    rng = np.random.default_rng(2)
    pos = (rng.random((10, 3))).astype(np.float32)
    spc = rng.choice(np.array(["Fe", "O"]), 10)
    write_sample(tmp_path, [(pos, spc)])
    # a species file holding the labels themselves (written outside the
    # sample's own directory in the reference)
    np.save(os.path.join(tmp_path, "atomic_species_1.npy"), spc)
    s = DiskSample(tmp_path)
    assert np.array_equal(s.load_chunk_species(1), spc)
    codes, labels = s.load_chunk_species(1, codes=True)
    assert np.array_equal(labels[codes], spc)
    np.save(os.path.join(tmp_path, "atomic_species_1.npy"), np.full(10, 7, np.uint8))
    try:
        s.load_chunk_species(1)
    except ValueError as e:
        assert "label table" in str(e)
    else:
        raise AssertionError("codes beyond the label table must raise")


def test_seeded_displacements_are_kept_and_unseeded_are_fresh():
    """A seeded thermal model displaces a chunk the same way on every load,
    so the displaced positions are kept; they equal thermal_displacement,
    a caller's copy cannot change them, and an unseeded model draws afresh."""
    from mosaic_gb300.sample import ChunkedSample, thermal_displacement
    rng = np.random.default_rng(3)
    pos = rng.uniform(-20, 20, (500, 3)).astype(np.float32)
    spc = np.array(["Cu"] * 500)
    th = dict(sigma=0.1, max_displacement=0.3, seed=7)
    s = ChunkedSample([(pos, spc), (pos[:200], spc[:200])], thermal=th)
    a = s.load_chunk_positions(2)
    want = thermal_displacement(pos[:200], 0.1, 0.3, 7, 2)
    assert np.array_equal(a, want)
    a += 1.0                                    # the caller's copy
    assert np.array_equal(s.load_chunk_positions(2), want)
    assert np.array_equal(s.load_chunk_positions(2, copy=False), want)
    assert np.array_equal(s.load_chunk_positions(1, raw=True), pos)
    s.thermal = dict(th, seed=8)                # another model: drawn again
    assert np.array_equal(s.load_chunk_positions(2), thermal_displacement(pos[:200], 0.1, 0.3, 8, 2))
    u = ChunkedSample([(pos, spc)], thermal=dict(sigma=0.1, max_displacement=0.3, seed=None))
    assert not np.array_equal(u.load_chunk_positions(1), u.load_chunk_positions(1))
