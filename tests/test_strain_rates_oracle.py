"""StrainRateComponents (RheologyDensity.c:2001-2097): the C restatement against the
reference compiled from its own sources (bit for bit), against the golden fixtures,
the drop-in over the CPU backend, and the arithmetic of a linear flow."""
import os

import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from golden import cases
from golden.make_golden import STRAIN_INPUTS, digest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
need_ref = pytest.mark.skipif(O.reference() is None, reason="reference build absent (oracle/_ref)")
need_shim = pytest.mark.skipif(O.shimtest() is None, reason="drop-in check library not built")

CASES = {
    # name: (builder, out_of_plane, compressible)
    "square": (lambda: W.velocity_field(seed=1, ncx=64), 0, 0.0),
    "air_compressible": (lambda: W.velocity_field(seed=2, ncx=57, ncz=41, air=0.3), 0, 1.0),
    "air_out_of_plane": (lambda: W.velocity_field(seed=3, ncx=40, ncz=66, air=0.2), 1, 1.0),
    "periodic_air": (lambda: W.velocity_field(seed=4, ncx=33, ncz=29, air=0.25, periodic=1), 1, 0.0),
    "fractional_compressible": (lambda: W.velocity_field(seed=5, ncx=20, ncz=21, air=0.1), 0, 0.37),
    "one_column": (lambda: W.velocity_field(seed=6, ncx=1, ncz=17), 1, 1.0),
    "one_row_periodic": (lambda: W.velocity_field(seed=7, ncx=19, ncz=1, periodic=1), 0, 1.0),
    "scaled": (lambda: W.velocity_field(seed=8, ncx=30, ncz=25, air=0.3, sc=W.TYPICAL), 1, 1.0),
    "near_overflow": (lambda: W.velocity_field(seed=9, ncx=20, ncz=20, air=0.2, v0=1e303, L=1e3), 1, 1.0),
    "subnormal": (lambda: W.velocity_field(seed=10, ncx=20, ncz=20, air=0.2, v0=3e-308, L=1e3), 1, 1.0),
}


def run(fn, w, oop, comp):
    a = {k: v.copy() for k, v in w.arrays.items()}
    assert fn(w.model, w.info["dx"], w.info["dz"], a, oop, comp) == R.MDZ_OK
    return a


def same_bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


@need_ref
@pytest.mark.parametrize("name", list(CASES))
def test_strain_rates_restatement_is_the_reference(name):
    make, oop, comp = CASES[name]
    w = make()
    a = run(O.ref_strain_rates, w, oop, comp)
    b = run(O.orc_strain_rates, w, oop, comp)
    for k in R.SR_N + R.SR_S:
        assert same_bits(a[k], b[k]), k


@pytest.mark.parametrize("name", list(cases.STRAIN_CASES))
def test_oracle_strain_rates_match_golden(name):
    builder, oop, comp = cases.STRAIN_CASES[name]
    w = builder()
    g = np.load(os.path.join(GOLDEN, f"strain_rates_{name}.npz"))
    assert str(g["inputs_sha256"]) == digest(w.arrays, STRAIN_INPUTS), "input generator changed"
    a = run(O.orc_strain_rates, w, oop, comp)
    for k in R.SR_N + R.SR_S:
        assert same_bits(a[k], g[k]), k


@need_shim
@pytest.mark.parametrize("name", ["air_out_of_plane", "periodic_air"])
def test_drop_in_strain_rates_match_reference(name):
    make, oop, comp = CASES[name]
    w = make()
    a = run(lambda *x: O.shim_strain_rates(*x, drop_in=False), w, oop, comp)
    b = run(lambda *x: O.shim_strain_rates(*x, drop_in=True), w, oop, comp)
    for k in R.SR_N + R.SR_S:
        assert same_bits(a[k], b[k]), k


def test_air_nodes():
    """Air cells and vertices get zeros, except wxz, which air vertices leave alone."""
    w = W.velocity_field(seed=9, ncx=30, ncz=30, air=0.3)
    a = run(O.orc_strain_rates, w, 1, 1.0)
    air_c = np.isin(a["BCp_type"], (30, 31))
    air_v = a["BCg_type"] == 30
    assert air_c.any() and air_v.any()
    for k in R.SR_N:
        assert np.all(a[k][air_c] == 0.0), k
    for k in ("exz", "exxd_s", "ezzd_s", "div_u_s"):
        assert np.all(a[k][air_v] == 0.0), k
    assert np.all(a["wxz"][air_v] == -7.0)
    assert np.all(a["wxz"][~air_v] != -7.0)


@pytest.mark.parametrize("oop,comp", [(0, 0.0), (0, 1.0), (1, 1.0)])
def test_linear_flow(oop, comp):
    """u = a x + b z, v = c x + d z: uniform rates away from air, to rounding."""
    ncx, ncz = 24, 18
    w = W.velocity_field(seed=10, ncx=ncx, ncz=ncz)
    dx, dz = w.info["dx"], w.info["dz"]
    ga, gb, gc, gd = 2e-15, -3e-15, 5e-16, -1.5e-15
    nx, nz = ncx + 1, ncz + 1
    xu, zu = np.arange(nx) * dx, (np.arange(nz + 1) - 0.5) * dz
    xv, zv = (np.arange(nx + 1) - 0.5) * dx, np.arange(nz) * dz
    w.arrays["u_in"] = (ga * xu[None, :] + gb * zu[:, None]).ravel()
    w.arrays["v_in"] = (gc * xv[None, :] + gd * zv[:, None]).ravel()
    a = run(O.orc_strain_rates, w, oop, comp)
    div = (ga + gd) * (1.0 + 0.5 * oop)
    expect_n = {"div_u": div, "exxd": ga - comp / 3.0 * div, "ezzd": gd - comp / 3.0 * div,
                "exz_n": 0.5 * (gb + gc), "wxz_n": 0.5 * (gc - gb)}
    for k, e in expect_n.items():
        assert np.allclose(a[k], e, rtol=1e-9, atol=1e-27), k
    for k, e in {"exz": 0.5 * (gb + gc), "wxz": 0.5 * (gc - gb), "exxd_s": expect_n["exxd"],
                 "ezzd_s": expect_n["ezzd"], "div_u_s": div}.items():
        assert np.allclose(a[k], e, rtol=1e-9, atol=1e-27), k
