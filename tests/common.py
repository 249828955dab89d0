"""Shared helpers of the parity tests: workload cloning and the parity measure.

Parity bar of the plain kernel against the reference: 1e-12 relative, with each
output measured against the natural magnitude of the quantity it belongs to.
The reference itself only resolves its local solve to |r/Eii| < 1e-13
(MDLIB/RheologyDensity.c:154,172), so an output that is a small difference of
larger quantities is only defined to that tolerance in the reference too:

  * strain-rate partition (eII_*, div_u_pl): scale max(|ref|, Eii of the node), the
    invariant the local solve normalises its residual by (for the anisotropic routine,
    that of its own effective strain rate, whose elastic term goes through the inverse of
    the anisotropic elastic matrix and can be tens of times the isotropic one);
  * dissipative viscosity eta_phys: scale |ref| * max(1, |ref| / eta_VE) (it is
    the reciprocal of the viscous + plastic part of Eii, ill-conditioned where
    deformation is mostly elastic);
  * dissipation Wdiss: scale max(|ref|, Wtot);
  * everything else: scale max(|ref|, 1e-3 max|field|) (signed fields near 0).

The eta_phys scale is formed from the node's averages.  Where one phase of a node is
near its yield stress, its plastic strain rate is a small difference whose last bits the
local solve's own tolerance leaves open, and its dissipative viscosity can dominate the
node's average while the averaged eta_VE hides it.  `eta_phys_phase_scale` forms the same
scale phase by phase (each phase's eta_phys and eta_VE from the oracle's ViscosityConcise
at that node), sum_p |d node / d eta_p| eta_p max(1, eta_p / eta_VE_p); the full-size
tests use it at the nodes the node-average scale flags.
"""
import numpy as np

import mdz_rheo as R
import oracle_lib as O

OUT_FIELDS = R.VER_INTERP + R.CEN_OUT + R.VER_OUT + ["phase_eta_n", "phase_eta_s"]
RTOL = 1e-12
ATOL_FRAC = 1e-3
PARTITION = {"eII_el", "eII_pl", "eII_pwl", "eII_exp", "eII_lin", "eII_gbs", "eII_cst", "div_u_pl"}


def clone(arrays):
    return {k: ([x.copy() for x in v] if isinstance(v, list) else v.copy()) for k, v in arrays.items()}


def field(a, k):
    v = a[k]
    return np.concatenate(v) if isinstance(v, list) else v


def node_strain_rates(a, model, where="n"):
    """Effective strain rates (Exx, Ezz, Exz) of the centroids ("n") or vertices ("s"): the
    strain rates plus the elastic stress memory, isotropic (RheologyDensity.c:1199-1204,
    :1335-1340) or, where the workload carries the anisotropy fields, through the inverse of
    the anisotropic elastic matrix (EffectiveStrainRate, RheologyDensity.c:116-146, called at
    AnisotropyRoutines.c:976, :1123)."""
    s = "_n" if where == "n" else "_s"
    if where == "n":
        exx, ezz, exz, sxx, szz, sxz, mu = (a["exxd"], a["ezzd"], a["exz_n"], a["sxxd0"], a["szzd0"],
                                            a["sxz0_n"], a["mu_n"])
    else:
        exx, ezz, exz, sxx, szz, sxz, mu = (a["exxd_s"], a["ezzd_s"], a["exz"], a["sxxd0_s"], a["szzd0_s"],
                                            a["sxz0"], a["mu_s"])
    if model.elastic != 1:
        return exx, ezz, exz
    eta_e = model.dt * mu
    if a.get("aniso_factor" + s) is None:
        return exx + sxx / eta_e / 2.0, ezz + szz / eta_e / 2.0, exz + sxz / eta_e / 2.0
    d1, d2, ani = a["d1" + s], a["d2" + s], 1.0 - 1.0 / a["aniso_factor" + s]
    D11, D12, D13 = 2.0 - 2.0 * ani * d1, 2.0 * ani * d1, -2.0 * ani * d2
    D22, D23, D33 = 2.0 - 2.0 * ani * d1, 2.0 * ani * d2, 1.0 + 2.0 * ani * (d1 - 0.5)
    a11, a12, a13 = D33 * D22 - D23 ** 2, D13 * D23 - D33 * D12, D12 * D23 - D13 * D22
    a22, a23, a33 = D33 * D11 - D13 ** 2, D12 * D13 - D11 * D23, D11 * D22 - D12 ** 2
    det = D11 * a11 + D12 * a12 + D13 * a13
    return (exx + (a11 / det * sxx + a12 / det * szz + a13 / det * sxz) / eta_e,
            ezz + (a12 / det * sxx + a22 / det * szz + a23 / det * sxz) / eta_e,
            exz + (a13 / det * sxx + a23 / det * szz + a33 / det * sxz) / eta_e / 2.0)


def node_Eii(a, model, where="n"):
    """Invariant of the effective strain rate of the centroids ("n") or vertices ("s"): the
    Eii that the node's local solves normalise their residual by (the anisotropic routine's
    rotation to the director frame leaves it unchanged)."""
    Exx, Ezz, Exz = node_strain_rates(a, model, where)
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


def eta_phys_phase_scale(w, ref, nodes, where="s", phases=False):
    """Per-node scale of eta_phys at centroid ("n") or vertex ("s") indices `nodes`, from
    every phase's dissipative viscosity eta_p and eta_VE_p (the oracle's ViscosityConcise
    on that node's inputs, prepared as NonNewtonianViscosityGrid prepares them:
    RheologyDensity.c:1199-1204, :1335-1340), combined by the model's phase average."""
    m, mat, a = w.model, w.mat, w.arrays
    nodes = np.asarray(nodes, np.int64)
    npn, np_ = nodes.size, mat.Nb_phases
    if npn == 0:
        return np.zeros(0)
    cen = where == "n"
    if cen:
        src = {"G": a["mu_n"], "T": a["T"], "P": a["p_in"], "d": a["d0_n"], "phi": a["phi0_n"], "X0": a["X0_n"],
               "Txx0": a["sxxd0"], "Tzz0": a["szzd0"], "Txz0": a["sxz0_n"], "strain_acc": a["strain_n"],
               "dil": a["dil_n"], "fric": a["fric_n"], "C": a["C_n"], "P0": a["p0_n"], "T0": a["T0_n"],
               "beta": a["bet_n"], "div": a["div_u"]}
    else:
        src = {"G": a["mu_s"], "T": ref["T_s"], "P": ref["P_s"], "d": ref["d0_s"], "phi": ref["phi0_s"],
               "X0": a["X0_s"], "Txx0": a["sxxd0_s"], "Tzz0": a["szzd0_s"], "Txz0": a["sxz0"],
               "strain_acc": a["strain_s"], "dil": a["dil_s"], "fric": a["fric_s"], "C": a["C_s"], "P0": a["p0_s"],
               "T0": np.zeros_like(a["mu_s"]), "beta": a["bet_s"], "div": a["div_u_s"]}
    pin = {k: np.repeat(v[nodes], np_) for k, v in src.items()}
    E = node_strain_rates(a, m, where)
    pin["Exx"], pin["Ezz"], pin["Exz"] = (np.repeat(x[nodes], np_) for x in E)
    aniso = a.get("aniso_factor_n") is not None
    if aniso:  # the director frame of NonNewtonianViscosityGridAniso (AnisotropyRoutines.c:959-961)
        s = "_n" if cen else "_s"
        angle = np.repeat(a["angle" + s][nodes], np_)
        lay = angle - np.pi / 2.0
        pin["lxlz"], pin["lx2"], pin["angle"] = np.cos(lay) * np.sin(lay), np.cos(lay) * np.cos(lay), angle
        pin["ani_fac"] = np.repeat(a["aniso_factor" + s][nodes], np_)
    pin["phase"] = np.tile(np.arange(np_, dtype=np.int32), npn)
    out = {k: np.zeros(npn * np_) for k in R.PT_OUT}
    pi, po = R.make_points(pin, out, centroid=1 if cen else 0)
    O.orc_points(m, mat, pi, po, npn * np_, 1 if aniso else 0)
    eta = out["eta"].reshape(npn, np_)
    eve = out["etaVE"].reshape(npn, np_)
    perc = np.stack([a["phase_perc_n" if cen else "phase_perc_s"][p][nodes] for p in range(np_)], axis=1)
    active = np.abs(perc) > 1e-13
    kappa = np.maximum(1.0, np.abs(eta / eve))
    if m.eta_average == 1:  # harmonic: node = 1 / sum perc / eta_p
        node = 1.0 / np.sum(np.where(active, perc / eta, 0.0), axis=1)
        terms = node[:, None] ** 2 * perc / np.abs(eta) * kappa
    elif m.eta_average == 2:  # geometric: node = exp(sum perc ln eta_p)
        node = np.exp(np.sum(np.where(active, perc * np.log(eta), 0.0), axis=1))
        terms = node[:, None] * np.abs(perc) * kappa
    else:  # arithmetic: node = sum perc eta_p
        terms = np.abs(perc * eta) * kappa
    scale = np.sum(np.where(active, terms, 0.0), axis=1)
    return (scale, eta, eve, perc) if phases else scale
