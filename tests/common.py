"""Shared helpers of the parity tests: workload cloning and the parity measure.

Parity bar of the plain kernel against the reference: 1e-12 relative, with each
output measured against the natural magnitude of the quantity it belongs to.
The reference itself only resolves its local solve to |r/Eii| < 1e-13
(MDLIB/RheologyDensity.c:154,172), so an output that is a small difference of
larger quantities is only defined to that tolerance in the reference too:

  * strain-rate partition (eII_*, div_u_pl): scale max(|ref|, Eii of the node);
  * dissipative viscosity eta_phys: scale |ref| * max(1, |ref| / eta_VE) (it is
    the reciprocal of the viscous + plastic part of Eii, ill-conditioned where
    deformation is mostly elastic);
  * dissipation Wdiss: scale max(|ref|, Wtot);
  * everything else: scale max(|ref|, 1e-3 max|field|) (signed fields near 0).
"""
import numpy as np

import mdz_rheo as R

OUT_FIELDS = R.VER_INTERP + R.CEN_OUT + R.VER_OUT + ["phase_eta_n", "phase_eta_s"]
RTOL = 1e-12
ATOL_FRAC = 1e-3
PARTITION = {"eII_el", "eII_pl", "eII_pwl", "eII_exp", "eII_lin", "eII_gbs", "eII_cst", "div_u_pl"}


def clone(arrays):
    return {k: ([x.copy() for x in v] if isinstance(v, list) else v.copy()) for k, v in arrays.items()}


def field(a, k):
    v = a[k]
    return np.concatenate(v) if isinstance(v, list) else v


def node_Eii(a, model, where="n"):
    """Effective strain-rate invariant of the centroids ("n") or vertices ("s")."""
    if where == "n":
        exx, ezz, exz, sxx, szz, sxz, mu = (a["exxd"], a["ezzd"], a["exz_n"], a["sxxd0"], a["szzd0"],
                                            a["sxz0_n"], a["mu_n"])
    else:
        exx, ezz, exz, sxx, szz, sxz, mu = (a["exxd_s"], a["ezzd_s"], a["exz"], a["sxxd0_s"], a["szzd0_s"],
                                            a["sxz0"], a["mu_s"])
    h = (0.5 / (model.dt * mu)) if model.elastic == 1 else 0.0
    Exx, Ezz, Exz = exx + sxx * h, ezz + szz * h, exz + sxz * h
    Eyy = -(Exx + Ezz)
    return np.sqrt(0.5 * (Exx ** 2 + Ezz ** 2 + Eyy ** 2) + Exz ** 2)


def scaled_error(x, ref, scale):
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.where(scale > 0, scale, 1.0)
    e = np.abs(x - ref) / den
    same = (x == ref) | (np.isnan(x) & np.isnan(ref))
    return np.where(same, 0.0, e)


def rel_err(x, ref, atol_frac=ATOL_FRAC):
    ref = np.asarray(ref, dtype=np.float64)
    fin = np.isfinite(ref)
    fmax = np.max(np.abs(ref[fin])) if np.any(fin) else 0.0
    return scaled_error(x, ref, np.maximum(np.abs(ref), atol_frac * fmax))


def worst(a, b, ref_arrays=None, model=None, fields=OUT_FIELDS):
    """{field: max scaled error} of a against reference b (see module doc)."""
    out = {}
    Eii_n = node_Eii(ref_arrays, model, "n") if ref_arrays is not None else None
    for k in fields:
        if k not in a or k not in b or a[k] is None or b[k] is None:
            continue
        x, ref = field(a, k), field(b, k)
        if ref.size == 0:
            out[k] = 0.0
            continue
        if k in PARTITION and Eii_n is not None:
            e = scaled_error(x, ref, np.maximum(np.abs(ref), Eii_n))
        elif k == "eta_phys_n":
            e = scaled_error(x, ref, np.abs(ref) * np.maximum(1.0, np.abs(ref) / np.abs(b["eta_n"])))
        elif k == "eta_phys_s":
            e = scaled_error(x, ref, np.abs(ref) * np.maximum(1.0, np.abs(ref) / np.abs(b["eta_s"])))
        elif k == "Wdiss":
            e = scaled_error(x, ref, np.maximum(np.abs(ref), np.abs(b["Wtot"])))
        else:
            e = rel_err(x, ref)
        out[k] = float(np.max(e))
    return out
