"""Shared helpers of the parity tests: workload cloning and error measures."""
import numpy as np

import mdz_rheo as R

OUT_FIELDS = R.VER_INTERP + R.CEN_OUT + R.VER_OUT + ["phase_eta_n", "phase_eta_s"]

# Parity bar of the plain kernel against the reference: 1e-12 relative.  Fields
# that are differences of nearly equal numbers (stress increments, signed
# components near zero) are judged against the field's own magnitude:
#   |gpu - ref| <= RTOL * max(|ref|, ATOL_FRAC * max|ref_field|)
RTOL = 1e-12
ATOL_FRAC = 1e-3


def clone(arrays):
    return {k: ([x.copy() for x in v] if isinstance(v, list) else v.copy()) for k, v in arrays.items()}


def field(a, k):
    v = a[k]
    return np.concatenate(v) if isinstance(v, list) else v


def rel_err(x, ref, atol_frac=ATOL_FRAC):
    """Per-element error scaled as in the parity bar (0 where both are equal)."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = np.max(np.abs(ref[np.isfinite(ref)])) if np.any(np.isfinite(ref)) else 0.0
    den = np.maximum(np.abs(ref), atol_frac * scale)
    den = np.where(den > 0, den, 1.0)
    e = np.abs(x - ref) / den
    same = (x == ref) | (np.isnan(x) & np.isnan(ref))
    return np.where(same, 0.0, e)


def worst(a, b, fields=OUT_FIELDS):
    """{field: max scaled error} over the fields present in both dicts."""
    out = {}
    for k in fields:
        if k in a and k in b and a[k] is not None and b[k] is not None:
            out[k] = float(np.max(rel_err(field(a, k), field(b, k)))) if field(b, k).size else 0.0
    return out
