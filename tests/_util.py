"""Shared helpers of the test suite: field comparisons and paired runs."""
import numpy as np


def rel_linf(a, b, floor):
    """max |a-b| / (|b| + floor) over the interior of two (nx+2, ny+2) fields."""
    a = np.asarray(a)[1:-1, 1:-1]
    b = np.asarray(b)[1:-1, 1:-1]
    return float(np.max(np.abs(a - b) / (np.abs(b) + floor)))


def phi_rel(a, b):
    a = np.asarray(a)[1:-1, 1:-1]
    b = np.asarray(b)[1:-1, 1:-1]
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def field_errors(g, r, n_zero):
    out = {f: rel_linf(g[f], r[f], n_zero) for f in ("ni", "ne", "nt")}
    out["ph"] = phi_rel(g["ph"], r["ph"])
    return out
