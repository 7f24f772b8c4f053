"""Atomic scattering tables: Waasmaier-Kirfel f0 and Cromer-Liberman f', f''.

Semantics follow the reference loaders (MOSAIC Beam.py:503-615):

* ``f0_WaasKirf.dat``: a ``#S <Z> <label>`` header opens an entry; a data line
  of exactly 11 numbers ``a1..a5 c b1..b5`` is stored as float32 under that
  label (a later line for the same label replaces it).
* ``f1f2_CromerLiberman.dat``: rows ``[E_eV, f', f'']`` under each header,
  stored as float32 (N, 3).
* f' + i f'' at energy E: linear interpolation between the bracketing rows,
  the first/last segment extended outside the table; the arithmetic runs on
  the float32 table values exactly as the reference does, so results are
  bit-identical.
* f0(0) = c + a1 + a2 + a3 + a4 + a5, summed left to right in float32.

The package bundles every f0 entry and the f', f'' tables of the common
elements (``data/dabax_subset.npz``, extracted by ``data/make_tables.py``).
Point ``MOSAIC_DABAX_DIR`` (or ``ScatteringTables(dabax_dir=...)``) at a DABAX
directory to use the complete files.
"""
from __future__ import annotations

import os
from functools import lru_cache

import numpy as np

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "dabax_subset.npz")


def parse_f0_file(path: str) -> dict:
    """label -> float32 (11,) Waasmaier-Kirfel row (Beam.py:503-526)."""
    rows, label = {}, None
    with open(path, "r") as fh:
        for line in fh:
            if line.startswith("#S"):
                label = line.split()[2].strip()
            elif not line.startswith("#") and label is not None:
                vals = line.split()
                if len(vals) == 11:
                    rows[label] = np.array([float(v) for v in vals], dtype=np.float32)
    return rows


def parse_f1f2_file(path: str) -> dict:
    """label -> float32 (N, 3) [E_eV, f', f''] (Beam.py:529-566)."""
    tables, label, acc = {}, None, []
    with open(path, "r") as fh:
        for line in fh:
            if line.startswith("#S"):
                if label is not None and acc:
                    tables[label] = np.array(acc, dtype=np.float32)
                label, acc = line.split()[2].strip(), []
            elif not line.startswith("#") and label is not None:
                vals = line.split()
                if len(vals) == 3:
                    acc.append([float(v) for v in vals])
    if label is not None and acc:
        tables[label] = np.array(acc, dtype=np.float32)
    return tables


def anomalous_at(energy_eV: float, table: np.ndarray) -> complex:
    """f' + i f'' at ``energy_eV`` (Beam.py:569-597), float32 arithmetic."""
    e = table[:, 0]
    i = int(np.searchsorted(e, energy_eV))
    i = min(max(i, 1), len(e) - 1)
    e0, e1 = e[i - 1], e[i]
    span = (e1 - e0) if e1 > e0 else 1e-20
    w = (energy_eV - e0) / span
    f1 = table[i - 1, 1] + (table[i, 1] - table[i - 1, 1]) * w
    f2 = table[i - 1, 2] + (table[i, 2] - table[i - 1, 2]) * w
    return complex(f1, f2)


def f0_at_zero(row: np.ndarray) -> float:
    """c + a1 + ... + a5 in float32, left to right (Beam.py:600-615)."""
    s = row[5]
    for i in range(5):
        s = s + row[i]
    return float(s)


def f0_value(row, s2):
    """Waasmaier-Kirfel f0 at s^2 = (sin(theta)/lambda)^2 in 1/A^2, float64."""
    row = np.asarray(row, dtype=np.float64)
    s2 = np.asarray(s2, dtype=np.float64)
    return row[5] + sum(row[i] * np.exp(-row[6 + i] * s2) for i in range(5))


class ScatteringTables:
    """f0 rows, f0(0) and f'+if'' per element label."""

    def __init__(self, dabax_dir: str | None = None):
        dabax_dir = dabax_dir or os.environ.get("MOSAIC_DABAX_DIR")
        if dabax_dir:
            self.f0 = parse_f0_file(os.path.join(dabax_dir, "f0_WaasKirf.dat"))
            self.f1f2 = parse_f1f2_file(os.path.join(dabax_dir, "f1f2_CromerLiberman.dat"))
            self.source = dabax_dir
        else:
            self.f0, self.f1f2 = _bundled()
            self.source = _DATA

    def has(self, label: str) -> bool:
        return str(label) in self.f0

    def row(self, label: str) -> np.ndarray:
        return self.f0[str(label)]

    def f0_zero(self, label: str) -> float:
        return f0_at_zero(self.f0[str(label)])

    def anomalous(self, label: str, energy_eV: float) -> complex:
        """f' + i f''; 0 for a label without an f1f2 table (as the reference's
        lookup does when ``db_f1f2.get`` misses, Beam.py:5683-5687)."""
        t = self.f1f2.get(str(label))
        if t is None:
            if str(label) in self.f0 and self.source == _DATA:
                raise KeyError(
                    f"no Cromer-Liberman f', f'' table for '{label}' in the bundled subset; "
                    "set MOSAIC_DABAX_DIR to a DABAX directory for the full tables")
            return 0j
        return anomalous_at(float(energy_eV), t)


@lru_cache(maxsize=1)
def _bundled():
    z = np.load(_DATA)
    f0 = {str(k): r.astype(np.float32) for k, r in zip(z["f0_keys"], z["f0_rows"])}
    f12, off = {}, 0
    for k, n in zip(z["f1f2_keys"], z["f1f2_len"]):
        f12[str(k)] = z["f1f2_rows"][off:off + int(n)].astype(np.float32)
        off += int(n)
    return f0, f12
