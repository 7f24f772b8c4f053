"""Chunked samples with the reference's chunk API: in memory
(``ChunkedSample``) and in the reference's on-disk format (``DiskSample``).

The scattering entry point reads a sample only through this duck type
(MOSAIC Sample.py:715-872): ``chunk_total``, ``chunk_atom_count(cid)``,
``load_chunk_positions(cid, use_gpu, raw)`` -> (N, 3) float32 Angstrom with
the thermal displacement applied on load, and ``load_chunk_species(cid,
use_gpu, codes)`` -> labels, or (codes, labels) with ``codes=True``.
Chunks are 1-based.

The Gaussian thermal displacement follows Sample.apply_temperature
(Sample.py:2084-2156, 2321-2334): one NumPy generator per chunk seeded with
SeedSequence([seed, chunk]), standard normals in the positions' dtype times
sigma, clipped to +-max_displacement when that is positive.
"""
from __future__ import annotations

import numpy as np


def thermal_displacement(positions, sigma, max_displacement=1.0, seed=40, chunk_number=None):
    """Displaced copy of ``positions`` (the reference's Gaussian rule)."""
    pos = np.asarray(positions)
    root = np.random.SeedSequence().entropy if seed is None else int(seed)
    key = [root] if chunk_number is None else [root, int(chunk_number)]
    rng = np.random.default_rng(np.random.SeedSequence(key))
    d = rng.standard_normal(size=pos.shape, dtype=pos.dtype)
    d *= float(sigma)
    if max_displacement is not None and max_displacement > 0.0:
        np.clip(d, -max_displacement, max_displacement, out=d)
    return pos + d


class ChunkedSample:
    """Chunks of (positions (N,3) Angstrom, species) held in host memory.

    Args:
        chunks: list of (positions, species) where species is an (N,) label
            array, or a (codes (N,) uint8/int, labels (S,)) pair.
        thermal: None or dict(sigma=, max_displacement=, seed=) for the
            Gaussian displacement applied on every load.
        dimensions: (Lx, Ly, Lz) in Angstrom (the sample box, informational).

    With a seed the displacement of a chunk is the same on every load, so
    the displaced positions are kept after the first (``keep_displaced``;
    they cost one more copy of the positions in host memory).
    """

    keep_displaced = True

    def __init__(self, chunks, thermal=None, dimensions=None, directory=""):
        self._chunks = []
        for pos, spc in chunks:
            pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
            if isinstance(spc, tuple):
                codes, labels = np.asarray(spc[0]), np.asarray(spc[1]).astype(str)
            else:
                labels, codes = np.unique(np.asarray(spc).astype(str), return_inverse=True)
                codes = codes.reshape(-1).astype(np.uint8 if labels.size <= 256 else np.uint16)
            if codes.shape[0] != pos.shape[0]:
                raise ValueError("positions/species size mismatch")
            self._chunks.append((pos, codes, labels))
        self._displaced = {}
        self.thermal = thermal
        self.directory = directory
        if dimensions is None and self._chunks:
            allp = [c[0] for c in self._chunks if c[0].size]
            if allp:
                lo = np.min([p.min(0) for p in allp], axis=0)
                hi = np.max([p.max(0) for p in allp], axis=0)
                dimensions = tuple((hi - lo).tolist())
        self.dimensions = dimensions

    @property
    def chunk_total(self):
        return len(self._chunks)

    def chunk_atom_count(self, chunk_number):
        return int(self._chunks[chunk_number - 1][0].shape[0])

    def load_chunk_positions(self, chunk_number, use_gpu=False, raw=False, copy=True):
        """The chunk's positions (A), thermally displaced when the sample has
        a thermal model (unless ``raw``); ``copy=False`` returns the stored
        array itself when no displacement applies (for readers that do not
        modify it)."""
        pos = self._chunks[chunk_number - 1][0]
        if self.thermal and not raw:
            t = self.thermal
            key = (t.get("sigma", 0.25), t.get("max_displacement", 1.0), t.get("seed", 40))
            if key[2] is None or not self.keep_displaced:     # fresh entropy on every load
                return thermal_displacement(pos, *key, chunk_number)
            kept = self._displaced.get(chunk_number)
            if kept is None or kept[0] != key:
                kept = (key, thermal_displacement(pos, *key, chunk_number))
                self._displaced[chunk_number] = kept
            return kept[1].copy() if copy else kept[1]
        return pos.copy() if copy else pos

    def load_chunk_species(self, chunk_number, use_gpu=False, codes=False):
        _, c, labels = self._chunks[chunk_number - 1]
        if codes:
            return c, labels
        return labels[c]

    @property
    def n_atoms(self):
        return sum(c[0].shape[0] for c in self._chunks)


class DiskSample:
    """A sample directory in the reference's on-disk format, read directly.

    Layout (Sample.py:543-676, 735-872): ``sample_metadata.json`` (with
    ``chunk_total`` and ``species_labels``), per chunk i (1-based)
    ``atomic_positions_{i}.npy`` (N, 3) Angstrom and ``atomic_species_{i}.npy``
    -- integer codes into ``species_labels``, or the labels themselves (files
    written outside the sample's own directory). Position files are opened
    memory-mapped; the atom count comes from the .npy header. The thermal
    displacement, when given (dict(sigma=, max_displacement=, seed=), the
    reference's ``temp_params`` for the Gaussian rule), is applied on every
    load, as the reference does, with the same per-chunk generator.
    """

    def __init__(self, directory, thermal=None):
        import json
        import os
        self.directory = str(directory)
        path = os.path.join(self.directory, "sample_metadata.json")
        with open(path) as fh:
            meta = json.load(fh)
        self.metadata = meta
        self._chunk_total = int(meta.get("chunk_total") or 0)
        self._labels = np.asarray(meta.get("species_labels") or [], dtype=str)
        self.thermal = thermal
        dims = meta.get("dimensions")
        self.dimensions = tuple(dims) if dims is not None else None

    def _path(self, stem, chunk_number):
        import os
        return os.path.join(self.directory, f"{stem}_{int(chunk_number)}.npy")

    @property
    def chunk_total(self):
        return self._chunk_total

    def chunk_atom_count(self, chunk_number):
        return int(np.load(self._path("atomic_positions", chunk_number), mmap_mode="r").shape[0])

    def load_chunk_positions(self, chunk_number, use_gpu=False, raw=False, copy=True):
        # every read is a fresh array: ``copy`` has nothing to do here
        pos = np.load(self._path("atomic_positions", chunk_number))
        if self.thermal and not raw:
            t = self.thermal
            return thermal_displacement(pos, t.get("sigma", 0.25), t.get("max_displacement", 1.0),
                                        t.get("seed", 40), chunk_number)
        return pos

    def load_chunk_species(self, chunk_number, use_gpu=False, codes=False):
        arr = np.load(self._path("atomic_species", chunk_number))
        if arr.dtype.kind in "iu":
            if arr.size and int(arr.max()) >= self._labels.size:
                raise ValueError(f"species codes in chunk {chunk_number} exceed the label table "
                                 f"({self._labels.size} labels) of sample_metadata.json")
            return (arr, self._labels) if codes else self._labels[arr]
        if codes:
            labels, inv = np.unique(arr.astype(str), return_inverse=True)
            return inv.reshape(-1).astype(np.uint8 if labels.size <= 256 else np.uint16), labels
        return arr.astype(str)

    @property
    def n_atoms(self):
        return sum(self.chunk_atom_count(c) for c in range(1, self._chunk_total + 1))


def write_sample(directory, chunks, labels=None, dimensions=None):
    """Write chunks in the on-disk format ``DiskSample`` reads: positions
    float32 and species codes (uint8, or uint16 above 256 labels) with the
    label table in ``sample_metadata.json``."""
    import json
    import os
    os.makedirs(directory, exist_ok=True)
    table = list(labels) if labels is not None else []
    for i, (pos, spc) in enumerate(chunks, start=1):
        labs, inv = np.unique(np.asarray(spc).astype(str), return_inverse=True)
        for lab in labs:
            if str(lab) not in table:
                table.append(str(lab))
        m = np.array([table.index(str(lab)) for lab in labs], dtype=np.int64)
        codes = m[inv.reshape(-1)].astype(np.uint8 if len(table) <= 256 else np.uint16)
        np.save(os.path.join(directory, f"atomic_positions_{i}.npy"),
                np.ascontiguousarray(pos, dtype=np.float32))
        np.save(os.path.join(directory, f"atomic_species_{i}.npy"), codes)
    meta = {"dimensions": None if dimensions is None else [float(v) for v in dimensions],
            "offset": None, "rotation": None, "chunk_total": len(chunks), "sample_type": None,
            "species_labels": table}
    with open(os.path.join(directory, "sample_metadata.json"), "w") as fh:
        json.dump(meta, fh, indent=4)
