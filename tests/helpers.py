"""Shared helpers of the test suite."""
import numpy as np
import torch

import oracle
from mosaic_gb300 import engine


def table_from_rows(wk_rows, f0z_rows, anom_rows):
    """SpeciesTable + per-atom species index from per-atom rows."""
    keys = [tuple(np.asarray(r, np.float32).tolist()) + (float(z), complex(a))
            for r, z, a in zip(wk_rows, f0z_rows, anom_rows)]
    uniq = sorted(set(keys), key=keys.index)
    idx = np.array([uniq.index(k) for k in keys], dtype=np.int32)
    wk = np.array([k[:11] for k in uniq], dtype=np.float32)
    f0z = np.array([k[11] for k in uniq], dtype=np.float32)
    an = np.array([k[12] for k in uniq], dtype=np.complex128)
    return engine.SpeciesTable([f"s{i}" for i in range(len(uniq))], wk, f0z, an), idx


def atoms_from_arrays(pos_m, idx, amp, table, device):
    amp = np.asarray(amp)
    a2 = np.stack([amp.real, amp.imag], 1).astype(np.float32) if np.iscomplexobj(amp) else \
        np.asarray(amp, np.float32).reshape(-1, 2)
    counts = np.bincount(idx, minlength=len(table.labels)).astype(np.int64)
    return engine.Atoms(torch.tensor(np.asarray(pos_m, np.float64).reshape(-1, 3), device=device),
                        torch.tensor(idx, dtype=torch.int32, device=device),
                        torch.tensor(a2, device=device), counts, table)


def field(out):
    engine.sync()
    return torch.view_as_complex(out).cpu().numpy()


def rel_max(a, ref):
    return float(np.abs(a - ref).max() / np.abs(ref).max())


def rel_intensity(a, ref):
    Ia, Ir = np.abs(a) ** 2, np.abs(ref) ** 2
    return float(np.abs(Ia - Ir).max() / Ir.max())


def kernel_case(d, i):
    """Case i of the reference's raw-kernel fixtures (kernel_cases.npz)."""
    p = f"c{i}_"
    ny, nz, rf, ap, dc, k, pdeg, ex, ey, ez = d[p + "meta"]
    return dict(pos=d[p + "pos_m"], wk=d[p + "wk"], f0z=d[p + "f0z"], anom=d[p + "anom"],
                amp=d[p + "amp"], cxyz=d[p + "cxyz"], ny=int(ny), nz=int(nz), rf=int(rf),
                ap=int(ap), dc=int(dc), k=float(k), pol=(pdeg, ex, ey, ez),
                cffi=d[p + "out_cffi"], numpy=d[p + "out_numpy"])


def run_case(c, device, fast, tile_atoms=128, dw=None, launch=None):
    """A kernel case on the GPU: the FP32 split sum (``fast``) or the FP64
    sum. ``dw`` (species index -> B [A^2]) sets Debye-Waller factors."""
    table, idx = table_from_rows(c["wk"], c["f0z"], c["anom"])
    if dw is not None:
        table.dw_b = np.array([float(dw(s)) for s in range(len(table.labels))], np.float32)
    atoms = atoms_from_arrays(c["pos"], idx, c["amp"], table, device)
    phys = engine.physics(c["k"], (1, 0, 0), c["ap"], c["pol"], c["dc"], c["rf"])
    pix = engine.Pixels(c["cxyz"], c["ny"], c["nz"], phys, device=device)
    if fast:
        tiles = engine.Tiles(atoms, c["k"], tile_atoms, device=device)
        out = engine.run_split(tiles, pix, phys, table, fresnel=1, launch=launch)
    else:
        out = engine.run_plain(atoms, pix, phys)
    return field(out)


def oracle_case(c, dw=None):
    """The oracle on a kernel case; ``dw`` as in ``run_case`` (per species of
    the case's unique factor rows)."""
    a = c["anom"]
    b = None
    if dw is not None:
        _, idx = table_from_rows(c["wk"], c["f0z"], c["anom"])
        b = np.array([float(dw(s)) for s in idx], np.float32)
    return oracle.scatter_f64(c["pos"], c["wk"], c["f0z"], a.real, a.imag, c["amp"].real,
                              c["amp"].imag, *c["cxyz"], c["k"], c["ny"], c["nz"], c["rf"],
                              c["ap"], c["pol"], c["dc"], dw_b=b)
