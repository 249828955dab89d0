"""UpdateParticleStress (RheologyParticles.c:1725-2004) on the CPU: the C restatement
against the reference compiled from its own sources (bit for bit: marker stresses,
directors and the rewritten wxz), against the golden fixtures, the drop-in over the CPU
backend, and the status of markers the reference cannot place."""
import os

import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from golden import cases
from golden.make_golden import load_marker_G, load_marker_inputs, marker_opts

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
need_ref = pytest.mark.skipif(O.reference() is None, reason="reference build absent (oracle/_ref)")
need_shim = pytest.mark.skipif(O.shimtest() is None, reason="drop-in check library not built")
OUT = ("sxxd", "szzd", "sxz", "nx", "nz")


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.array_equal(a.view(np.uint64), b.view(np.uint64)) if a.dtype == np.float64 else np.array_equal(a, b)


def run(fn, w, opts):
    grid = {k: v.copy() for k, v in w.arrays.items()}
    mk = {k: v.copy() for k, v in w.info["markers"].items()}
    rc = fn(w.model, opts, grid, mk, w.info["dx"], w.info["dz"])
    return rc, grid, mk


def boundary_workload():
    """Markers exactly on vertex and centroid coordinates, on the domain edges and at its
    corners: the cell and weight arithmetic must place them as the reference does."""
    w = W.marker_workload(seed=70, ncx=40, ncz=30, markers_per_cell=2, air=0.2, periodic=1)
    mk = w.info["markers"]
    xg, zg, xc, zc = w.arrays["xg_coord"], w.arrays["zg_coord"], w.arrays["xvz_coord"], w.arrays["zvx_coord"]
    rng = np.random.default_rng(1)
    pick = rng.choice(mk["x"].size, 600, replace=False)
    mk["x"][pick[:150]] = rng.choice(xg, 150)
    mk["z"][pick[150:300]] = rng.choice(zg, 150)
    mk["x"][pick[300:450]] = rng.choice(xc[1:-1], 150)
    mk["z"][pick[450:600]] = rng.choice(zc[1:-1], 150)
    mk["x"][:4] = [xg[0], xg[-1], xg[0], xg[-1]]
    mk["z"][:4] = [zg[0], zg[0], zg[-1], zg[-1]]
    return w


def tiny_weight_workload():
    """Markers at the edge of their nearest vertex's support in both axes: P2Mastah
    weights of magnitude 1e-31 to 1e-29, negative (one ulp past the edge once rounded)
    or positive, below the 1e-30 threshold but not zero, at vertices few other active
    markers reach -- the exact weight sums decide wxz there."""
    w = W.marker_workload(seed=71, ncx=24, ncz=18, markers_per_cell=2, air=0.2)
    mk = w.info["markers"]
    xg, zg, dx, dz = w.arrays["xg_coord"], w.arrays["zg_coord"], w.info["dx"], w.info["dz"]
    rng = np.random.default_rng(2)
    mk["phase"][rng.random(mk["phase"].size) < 0.9] = -1
    n = 40
    jx, iz = rng.integers(1, xg.size - 2, n), rng.integers(1, zg.size - 2, n)
    hx, hz = dx / 2, dz / 2
    mk["x"][:n] = np.nextafter(xg[jx] + hx, xg[jx])
    mk["z"][:n] = np.nextafter(zg[iz] + hz, zg[iz])
    mk["x"][n // 2:n] = xg[jx[n // 2:]] + hx * (1 - 2.0 ** -51)
    mk["z"][n // 2:n] = zg[iz[n // 2:]] + hz * (1 - 2.0 ** -51)
    mk["phase"][:n] = 0
    return w


CASES = {
    # name: (builder, elastic, stress_rotation, anisotropy, advection, interp_stencil)
    "jaumann": (lambda: W.marker_workload(seed=1, ncx=31, ncz=24), 1, 1, 0, 1, 1),
    "analytical_director": (lambda: W.marker_workload(seed=2, ncx=27, ncz=30, air=0.3), 1, 2, 1, 1, 1),
    "periodic_stencil9_director": (lambda: W.marker_workload(seed=3, ncx=25, ncz=19, markers_per_cell=9,
                                                             air=0.2, periodic=1), 1, 1, 1, 1, 9),
    "no_rotation": (lambda: W.marker_workload(seed=4, ncx=20, ncz=22, air=0.25), 1, 0, 0, 1, 1),
    "elastic_off_director": (lambda: W.marker_workload(seed=5, ncx=18, ncz=21, periodic=1), 0, 1, 1, 1, 1),
    "no_advection": (lambda: W.marker_workload(seed=6, ncx=19, ncz=17, air=0.3), 1, 1, 1, 0, 9),
    "typical_scale_dense": (lambda: W.marker_workload(seed=7, ncx=16, ncz=16, markers_per_cell=16, sc=W.TYPICAL),
                            1, 2, 1, 1, 1),
    "one_column_of_cells": (lambda: W.marker_workload(seed=8, ncx=1, ncz=9, markers_per_cell=6), 1, 1, 1, 1, 1),
    "markers_on_boundaries": (boundary_workload, 1, 1, 1, 1, 9),
    "tiny_weights": (tiny_weight_workload, 1, 1, 0, 1, 1),
    # subgrid_diffusion 2, the last element
    "subgrid2_jaumann_air": (lambda: W.marker_workload(seed=12, ncx=23, ncz=19, air=0.2), 1, 1, 0, 1, 1, 2),
    "subgrid2_periodic_stencil9_director": (lambda: W.marker_workload(seed=13, ncx=21, ncz=17, markers_per_cell=9,
                                                                      periodic=1, air=0.15), 1, 2, 1, 1, 9, 2),
    "subgrid2_typical_scale": (lambda: W.marker_workload(seed=14, ncx=16, ncz=18, markers_per_cell=8, sc=W.TYPICAL),
                               1, 0, 0, 1, 1, 2),
    "subgrid2_markers_on_boundaries": (boundary_workload, 1, 1, 0, 1, 9, 2),
    "subgrid2_tiny_weights": (tiny_weight_workload, 1, 1, 0, 1, 1, 2),
    "subgrid2_one_column_of_cells": (lambda: W.marker_workload(seed=15, ncx=1, ncz=9, markers_per_cell=6),
                                     1, 1, 0, 1, 9, 2),
}


def opts_of(name, w):
    return marker_opts(*CASES[name][1:], G=w.info["G"])


@need_ref
@pytest.mark.parametrize("name", list(CASES))
def test_marker_stress_restatement_is_the_reference(name):
    w = CASES[name][0]()
    opts = opts_of(name, w)
    ra, ga, ma = run(O.ref_marker_stress, w, opts)
    rb, gb, mb = run(O.orc_marker_stress, w, opts)
    assert ra == 0 and rb == R.MDZ_OK
    for k in OUT:
        assert same(ma[k], mb[k]), k
    assert same(ga["wxz"], gb["wxz"])
    if opts.elastic == 1:
        assert np.any(ma["sxxd"] != w.info["markers"]["sxxd"]) and np.any(ga["wxz"] != w.arrays["wxz"])


@pytest.mark.parametrize("name", list(cases.MARKER_CASES))
def test_oracle_marker_stress_matches_golden(name):
    g = np.load(os.path.join(GOLDEN, f"markers_{name}.npz"))
    model, grid, mk, dx, dz = load_marker_inputs(g)
    opts = marker_opts(*cases.MARKER_CASES[name][1:], G=load_marker_G(g))
    assert O.orc_marker_stress(model, opts, grid, mk, dx, dz) == R.MDZ_OK
    for k in OUT:
        assert same(mk[k], g["out_" + k]), k
    assert same(grid["wxz"], g["out_wxz"])


@need_shim
@pytest.mark.parametrize("name", ["analytical_director", "periodic_stencil9_director",
                                  "subgrid2_periodic_stencil9_director"])
def test_drop_in_marker_stress_matches_reference(name):
    w = CASES[name][0]()
    opts = opts_of(name, w)
    _, ga, ma = run(lambda *a: O.shim_marker_stress(*a, drop_in=False), w, opts)
    _, gb, mb = run(lambda *a: O.shim_marker_stress(*a, drop_in=True), w, opts)
    for k in OUT:
        assert same(ma[k], mb[k]), k
    assert same(ga["wxz"], gb["wxz"])


def test_unchanged_grid_stress_leaves_markers():
    """No stress change on the grid and no rotation: every marker keeps its stress, and
    the director stays a unit vector."""
    w = W.marker_workload(seed=9, ncx=20, ncz=20, air=0.2)
    w.arrays["sxxd0"], w.arrays["szzd0"], w.arrays["sxz0"] = (w.arrays["sxxd"].copy(), w.arrays["szzd"].copy(),
                                                              w.arrays["sxz"].copy())
    rc, g, mk = run(O.orc_marker_stress, w, marker_opts(1, 0, 1, 1, 1))
    assert rc == R.MDZ_OK
    for k in ("sxxd", "szzd", "sxz"):
        assert np.array_equal(mk[k], w.info["markers"][k]), k
    act = mk["phase"] != -1
    assert np.allclose(np.hypot(mk["nx"][act], mk["nz"][act]), 1.0, rtol=0, atol=4e-16)


def test_marker_beyond_grid_and_subgrid_diffusion_status():
    w = W.marker_workload(seed=10, ncx=12, ncz=10)
    w.info["markers"]["x"][5] = w.arrays["xg_coord"][-1] + 0.7 * w.info["dx"]
    rc, _, _ = run(O.orc_marker_stress, w, marker_opts(1, 1, 0, 1, 1))
    assert rc == R.MDZ_EMARKER_OUT
    rc, _, _ = run(O.orc_marker_stress, w, marker_opts(1, 1, 0, 1, 1, 2, G=w.info["G"]))
    assert rc == R.MDZ_EMARKER_OUT
    w = W.marker_workload(seed=11, ncx=8, ncz=8)
    rc, _, _ = run(O.orc_marker_stress, w, marker_opts(1, 1, 0, 1, 1, 2))  # no shear modulus
    assert rc == R.MDZ_EINVAL
    w.info["markers"]["phase"][3] = 3  # a phase the model does not have
    rc, _, _ = run(O.orc_marker_stress, w, marker_opts(1, 1, 0, 1, 1, 2, G=w.info["G"]))
    assert rc == R.MDZ_EINVAL
    w.info["markers"]["phase"][3] = 0
    w.arrays["eta_phys_s"][:] = 0.0  # zero Maxwell time: exp(-inf) = 0, a full relaxation, still finite
    rc, _, _ = run(O.orc_marker_stress, w, marker_opts(1, 1, 0, 1, 1, 2, G=w.info["G"]))
    assert rc == R.MDZ_OK


@pytest.mark.parametrize("stencil", [1, 9])
def test_subgrid_diffusion_without_relaxation_is_the_plain_update(stencil):
    """With Maxwell times so long that exp(-dt/t) rounds to 1, the subgrid increments
    are zero, P2Mastah brings zeros to the grid, and what comes back is the grid's whole
    increment: the update of subgrid_diffusion 0, bit for bit."""
    w = W.marker_workload(seed=16, ncx=19, ncz=15, air=0.2, periodic=1)
    w.arrays["eta_phys_s"][:] = 1e40
    r0, g0, m0 = run(O.orc_marker_stress, w, marker_opts(1, 1, 1, 1, stencil))
    r2, g2, m2 = run(O.orc_marker_stress, w, marker_opts(1, 1, 1, 1, stencil, 2, G=w.info["G"]))
    assert r0 == r2 == R.MDZ_OK
    for k in OUT:
        assert same(m0[k], m2[k]), k
    assert same(g0["wxz"], g2["wxz"])
