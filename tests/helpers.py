"""Shared helpers of the test suite."""
import numpy as np
import torch

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
