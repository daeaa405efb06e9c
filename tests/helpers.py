"""Shared comparison helpers for the parity tests."""
import numpy as np

CONS_NAMES = ("mass", "px", "py", "pz", "energy")


def rel_err(a, b):
    """Norm-wise relative error max|a-b| / max|b| (absolute when b is all zero)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.max(np.abs(b)) if b.size else 0.0
    d = np.max(np.abs(a - b)) if b.size else 0.0
    return float(d / scale) if scale > 0 else float(d)


def compare_cells(got, ref, fields=("cons", "prim", "grad", "extrap", "facc", "dt", "v_rel"), rows=True):
    """Per-field (and per-row) norm-wise relative errors between two Cells."""
    out = {}
    for f in fields:
        a, b = getattr(got, f), getattr(ref, f)
        if rows and a.ndim == 2:
            for k in range(a.shape[0]):
                out[f"{f}[{k}]"] = rel_err(a[k], b[k])
        else:
            out[f] = rel_err(a, b)
    out["timebin"] = float(np.max(np.abs(got.timebin.astype(np.int64) - ref.timebin.astype(np.int64))))
    return out


def totals(cells, mesh=None):
    """Sum of conserved quantities including pending fluxes (space.rs:1248-1270)."""
    return (cells.cons + cells.facc).sum(axis=1)
