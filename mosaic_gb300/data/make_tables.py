"""Extract the bundled scattering-table subset from DABAX files.

    python mosaic_gb300/data/make_tables.py <dir with f0_WaasKirf.dat and f1f2_CromerLiberman.dat>

Writes ``dabax_subset.npz`` beside this script: every Waasmaier-Kirfel f0 row
(11 float32 per entry, neutral atoms and ions) and the Cromer-Liberman
[E, f', f''] rows (float32) of the elements in ``F1F2_ELEMENTS``. The same
parser as the runtime (``mosaic_gb300.tables``) reads the files, so the
bundled arrays are bit-identical to parsing the full files.
"""
from __future__ import annotations

import os
import sys

import numpy as np

F1F2_ELEMENTS = [
    "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S",
    "Cl", "Ar", "K", "Ca", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge",
    "As", "Se", "Sr", "Zr", "Nb", "Mo", "Ag", "Cd", "In", "Sn", "Sb", "Te", "Ba", "Ta",
    "W", "Pt", "Au", "Pb"]


def main(src_dir: str) -> None:
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(os.path.dirname(here)))
    from mosaic_gb300.tables import parse_f0_file, parse_f1f2_file

    f0 = parse_f0_file(os.path.join(src_dir, "f0_WaasKirf.dat"))
    f12 = parse_f1f2_file(os.path.join(src_dir, "f1f2_CromerLiberman.dat"))
    keys = sorted(f0)
    sel = [e for e in F1F2_ELEMENTS if e in f12]
    arrays = {"f0_keys": np.array(keys), "f0_rows": np.stack([f0[k] for k in keys]),
              "f1f2_keys": np.array(sel),
              "f1f2_len": np.array([f12[e].shape[0] for e in sel], dtype=np.int64),
              "f1f2_rows": np.concatenate([f12[e] for e in sel]).astype(np.float32)}
    np.savez_compressed(os.path.join(here, "dabax_subset.npz"), **arrays)
    print(f"{len(keys)} f0 entries, {len(sel)} f1f2 tables")


if __name__ == "__main__":
    main(sys.argv[1])
