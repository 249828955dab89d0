"""GPU parity against the golden fixtures of MDOODZ7.0's own code (grids and the
feature point cases), with the parity measure of tests/common.py."""
import os

import numpy as np
import pytest

import mdz_rheo as R
from common import RTOL, rel_err, scaled_error, worst
from golden import cases
from golden.make_golden import grid_outputs

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ctx():
    c = R.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", list(cases.GRID_CASES))
def test_gpu_grid_matches_golden(ctx, name):
    builder, aniso, fu = cases.GRID_CASES[name]
    w = builder()
    inputs = {k: (list(v) if isinstance(v, list) else v.copy()) for k, v in w.arrays.items()}
    fn = ctx.sweep_aniso if aniso else ctx.sweep
    rc, st = fn(w.model, w.mat, R.FieldSet(w.arrays), final_update=fu, check=False)
    assert rc == R.MDZ_OK
    g = np.load(os.path.join(GOLDEN, f"grid_{name}.npz"))
    ref = {k: g[k] for k in g.files if k != "inputs_sha256"}
    got = grid_outputs(w.arrays)
    errs = worst(got, ref, inputs, w.model, fields=list(ref))
    print(name, {k: f"{v:.1e}" for k, v in errs.items() if v > 1e-15})
    assert max(errs.values()) <= RTOL, errs


def point_scales(k, ref, pin, md):
    """Natural magnitude of each ViscosityConcise output (see tests/common.py)."""
    Exx, Ezz, Exz = pin["Exx"], pin["Ezz"], pin["Exz"]
    Eii = np.sqrt(0.5 * (Exx ** 2 + Ezz ** 2 + (Exx + Ezz) ** 2) + Exz ** 2)
    a = np.abs(ref[k])
    if k.startswith("Eii_") or k == "div_pl":
        return np.maximum(a, Eii)
    if k == "eta":
        return a * np.maximum(1.0, a / np.abs(ref["etaVE"]))
    if k == "Wdiss":
        return np.maximum(a, np.abs(ref["Wtot"]))
    if k == "OverS":
        return np.maximum(a, 2.0 * np.abs(ref["etaVE"]) * Eii)
    if k == "div_el":
        return np.maximum(a, (np.abs(ref["Pcorr"]) + np.abs(pin["P0"])) * pin["beta"] / md.dt)
    fin = np.isfinite(ref[k])
    fmax = np.max(a[fin]) if np.any(fin) else 0.0
    return np.maximum(a, 1e-3 * fmax)


@pytest.mark.parametrize("name", list(cases.POINT_CASES))
def test_gpu_points_match_golden(ctx, name):
    md, m, pin, aniso, centroid, fu = cases.point_case(name)
    n = pin["phase"].size
    out = cases.alloc_point_outputs(n)
    pi, po = R.make_points(pin, out, centroid=centroid, final_update=fu)
    assert ctx.points(md, m, pi, po, n, aniso=int(aniso)) == R.MDZ_OK
    assert np.all(out["status"] == 0)
    g = np.load(os.path.join(GOLDEN, f"points_{name}.npz"))
    ref = {k: g[k] for k in R.PT_OUT}
    errs = {}
    for k in R.PT_OUT:
        errs[k] = float(np.max(scaled_error(out[k], ref[k], point_scales(k, ref, pin, md))))
    print(name, {k: f"{v:.1e}" for k, v in errs.items() if v > 1e-15})
    assert max(errs.values()) <= RTOL, errs
