"""The sweep's input preparation on the CPU: CohesionFrictionDilationGrid / Softening
(RheologyDensity.c:1432-1628) and ShearModCompExpGrid (:1634-1755).

The restatement (oracle/rheo_oracle.c) is fed the plastic strain that the reference's
own marker interpolation (P2Mastah) puts on the grid, and must equal the reference's
whole CohesionFrictionDilationGrid bit for bit; ShearModCompExpGrid likewise.  Then the
golden fixtures, the drop-in over the CPU backend and the error status."""
import os
import platform

import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from common import clone
from golden import cases
from golden.make_golden import load_prep_inputs, prep_inputs_digest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
need_ref = pytest.mark.skipif(O.reference() is None, reason="reference build absent (oracle/_ref)")
need_shim = pytest.mark.skipif(O.shimtest() is None, reason="drop-in check library not built")


def same_bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


SOFT = {
    # name: (builder, smooth_softening, hardening_modulus, marker_noise, interp_stencil)
    "piecewise": (lambda: W.prep_workload(seed=1, ncx=40, ncz=31, nphases=5, markers_per_cell=5), 0, 0, 0, 1),
    "piecewise_air_periodic_noise": (lambda: W.prep_workload(seed=2, ncx=37, ncz=29, nphases=4, air=0.3,
                                                            periodic=1, markers_per_cell=5), 0, 0, 1, 1),
    "erfc_air": (lambda: W.prep_workload(seed=3, ncx=30, ncz=33, nphases=3, air=0.2, markers_per_cell=5), 1, 0, 0, 1),
    "erfc_noise_stencil9": (lambda: W.prep_workload(seed=4, ncx=28, ncz=25, nphases=4, markers_per_cell=8), 1, 0, 1, 9),
    "hardening": (lambda: W.prep_workload(seed=5, ncx=33, ncz=20, nphases=2, air=0.25, markers_per_cell=5), 0, 1, 0, 1),
    "hardening_wins_over_erfc": (lambda: W.prep_workload(seed=6, ncx=21, ncz=22, nphases=3, markers_per_cell=5), 1, 1, 1, 1),
    "one_phase_typical_scale": (lambda: W.prep_workload(seed=7, ncx=26, ncz=19, nphases=1, sc=W.TYPICAL,
                                                       markers_per_cell=5), 0, 0, 1, 1),
}


@need_ref
@pytest.mark.parametrize("name", list(SOFT))
def test_softening_restatement_is_the_reference(name):
    make, smooth, hard, noise, stencil = SOFT[name]
    w = make()
    mk = dict(w.info["markers"], interp_stencil=stencil)
    a, b = clone(w.arrays), clone(w.arrays)
    rc, sn, ss = O.ref_softening_markers(w.model, w.mat, R.PrepFieldSet(a), mk, smooth, hard, noise)
    assert rc == 0 and np.any(sn > 0)
    b["strain_pl_n"], b["strain_pl_s"] = sn, ss
    assert O.orc_softening(w.model, w.mat, R.PrepFieldSet(b), smooth, hard, noise) == R.MDZ_OK
    for k in R.SOFT_N + R.SOFT_S:
        assert same_bits(a[k], b[k]), k


SHEAR = {
    "basic": lambda: W.prep_workload(seed=11, ncx=40, ncz=30, nphases=5),
    "air_periodic": lambda: W.prep_workload(seed=12, ncx=35, ncz=28, nphases=4, air=0.3, periodic=1),
    "one_phase_typical": lambda: W.prep_workload(seed=13, ncx=20, ncz=31, nphases=1, sc=W.TYPICAL),
    "periodic_one_column_of_cells": lambda: W.prep_workload(seed=14, ncx=1, ncz=12, nphases=3, periodic=1),
}


@need_ref
@pytest.mark.parametrize("name", list(SHEAR))
def test_shear_modulus_restatement_is_the_reference(name):
    w = SHEAR[name]()
    a, b = clone(w.arrays), clone(w.arrays)
    assert O.ref_shear_modulus(w.model, w.mat, R.PrepFieldSet(a)) == 0
    assert O.orc_shear_modulus(w.model, w.mat, R.PrepFieldSet(b)) == R.MDZ_OK
    for k in R.MOD_N + R.MOD_S:
        assert same_bits(a[k], b[k]), k


def golden_prep(name, kind):
    """A preparation fixture: its stored inputs (as a workload) and the reference's outputs."""
    g = np.load(os.path.join(GOLDEN, f"{kind}_{name}.npz"))
    model, mat, arrays = load_prep_inputs(g)
    return W.Workload(kind, model, mat, arrays), g


@pytest.mark.skipif(platform.machine() != "x86_64", reason="the fixtures were generated on an x86-64 host")
@pytest.mark.parametrize("kind,name", [("softening", n) for n in cases.SOFTENING_CASES]
                         + [("shear_modulus", n) for n in cases.SHEAR_CASES])
def test_prep_fixture_inputs_are_the_generators(kind, name):
    """On the host that made them, the stored inputs are what the case generators give."""
    builder = cases.SOFTENING_CASES[name][0] if kind == "softening" else cases.SHEAR_CASES[name]
    g = np.load(os.path.join(GOLDEN, f"{kind}_{name}.npz"))
    assert str(g["inputs_sha256"]) == prep_inputs_digest(builder()), "input generator changed"


@pytest.mark.parametrize("name", list(cases.SOFTENING_CASES))
def test_oracle_softening_matches_golden(name):
    w, g = golden_prep(name, "softening")
    _, smooth, hard, noise, _ = cases.SOFTENING_CASES[name]
    assert O.orc_softening(w.model, w.mat, R.PrepFieldSet(w.arrays), smooth, hard, noise) == R.MDZ_OK
    for k in R.SOFT_N + R.SOFT_S:
        assert same_bits(w.arrays[k], g[k]), k


@pytest.mark.parametrize("name", list(cases.SHEAR_CASES))
def test_oracle_shear_modulus_matches_golden(name):
    w, g = golden_prep(name, "shear_modulus")
    assert O.orc_shear_modulus(w.model, w.mat, R.PrepFieldSet(w.arrays)) == R.MDZ_OK
    for k in R.MOD_N + R.MOD_S:
        assert same_bits(w.arrays[k], g[k]), k


@need_shim
@pytest.mark.parametrize("name", ["piecewise_air_periodic_noise", "erfc_air"])
def test_drop_in_softening_matches_reference(name):
    """The drop-in CohesionFrictionDilationGrid runs the reference's P2Mastah itself, then
    the library; against the reference's function on the same grid and markers."""
    make, smooth, hard, noise, stencil = SOFT[name]
    w = make()
    mk = dict(w.info["markers"], interp_stencil=stencil)
    a, b = clone(w.arrays), clone(w.arrays)
    O.shim_softening_markers(w.model, w.mat, R.PrepFieldSet(a), mk, smooth, hard, noise, drop_in=False)
    O.shim_softening_markers(w.model, w.mat, R.PrepFieldSet(b), mk, smooth, hard, noise, drop_in=True)
    for k in R.SOFT_N + R.SOFT_S:
        assert same_bits(a[k], b[k]), k


@need_shim
def test_drop_in_shear_modulus_matches_reference():
    w = SHEAR["air_periodic"]()
    a, b = clone(w.arrays), clone(w.arrays)
    O.shim_shear_modulus(w.model, w.mat, R.PrepFieldSet(a), drop_in=False)
    O.shim_shear_modulus(w.model, w.mat, R.PrepFieldSet(b), drop_in=True)
    for k in R.MOD_N + R.MOD_S:
        assert same_bits(a[k], b[k]), k


def test_shear_modulus_infinite_status():
    """A solid centroid with no phase present has an infinite harmonic modulus: the
    reference exits with code 32, the restatement returns MDZ_ESHEAR_INF."""
    w = W.prep_workload(seed=15, ncx=10, ncz=8, nphases=2)
    for p in range(2):
        w.arrays["phase_perc_n"][p][17] = 0.0
    assert O.orc_shear_modulus(w.model, w.mat, R.PrepFieldSet(w.arrays)) == R.MDZ_ESHEAR_INF
    assert np.isinf(w.arrays["mu_n"][17])


def test_softening_piecewise_values():
    """Style 0 against its definition on one phase: constant below pls_start, linear in
    between, the end value from pls_end on."""
    w = W.prep_workload(seed=16, ncx=30, ncz=30, nphases=1)
    m = w.mat
    m.phi_soft[0] = m.psi_soft[0] = m.coh_soft[0] = 1
    s = w.arrays["strain_pl_n"]
    O.orc_softening(w.model, m, R.PrepFieldSet(w.arrays))
    lo, hi = m.pls_start[0], m.pls_end[0]
    expect = np.where(s < lo, m.phi[0], np.where(s >= hi, m.phi_end[0],
                                                 m.phi[0] + (m.phi_end[0] - m.phi[0]) / (hi - lo) * s))
    assert np.allclose(w.arrays["fric_n"], expect, rtol=1e-15, atol=0)
    assert np.any(s == lo) and np.any(s == hi)
