"""The MDOODZ-side drop-in (mdoodz7.0_gb300/host/mdz_rheo_mdoodz.c) on the CPU.

The drop-in defines NonNewtonianViscosityGrid / NonNewtonianViscosityGridAniso with
the reference's signatures and unpacks `grid`, `mat_prop`, `params` and `scale` into
the library's structs.  Here it runs over a CPU backend (oracle/shim_backend.c, the C
restatement) on a real `grid` built by the reference harness, side by side with the
reference's own function compiled from its sources; every output must agree bit for
bit, which pins the unpacking of every field.  Needs the reference tree (build host).
"""
import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from common import OUT_FIELDS, clone, field

pytestmark = pytest.mark.skipif(O.shimtest() is None, reason="drop-in check library not built (needs the reference tree)")

CASES = {
    "plain_small": (lambda: W.plain_small(seed=0, ncx=41), False, 0),
    "plain_large": (lambda: W.plain_large(seed=1, ncx=40, ncz=36), False, 0),
    "plain_large_final_update": (lambda: W.plain_large(seed=2, ncx=33), False, 1),
    "plain_large_harmonic_typical": (lambda: W.plain_large(seed=3, ncx=30, sc=W.TYPICAL, eta_average=1), False, 0),
    "aniso": (lambda: W.aniso(seed=4, ncx=32), True, 0),
}


@pytest.mark.parametrize("name", list(CASES))
def test_drop_in_matches_reference(name):
    make, aniso, fu = CASES[name]
    w = make()
    a, b = clone(w.arrays), clone(w.arrays)
    assert O.shim_sweep(w.model, w.mat, R.FieldSet(a), fu, aniso, drop_in=False) == 0
    assert O.shim_sweep(w.model, w.mat, R.FieldSet(b), fu, aniso, drop_in=True) == 0
    n = 0
    for k in OUT_FIELDS + (["VE_s", "VE_n"] if aniso else []):
        if a.get(k) is None:
            continue
        x, y = field(b, k), field(a, k)
        assert np.array_equal(x, y, equal_nan=True), k
        n += 1
    assert n >= 30


def test_periodic_and_air():
    w = W.plain_large(seed=5, ncx=24)
    w.model.periodic_x = 1
    w.arrays["BCp_type"][-48:] = 30
    w.arrays["BCg_type"][-25 * 3:] = 30
    a, b = clone(w.arrays), clone(w.arrays)
    O.shim_sweep(w.model, w.mat, R.FieldSet(a), 0, False, drop_in=False)
    O.shim_sweep(w.model, w.mat, R.FieldSet(b), 0, False, drop_in=True)
    for k in OUT_FIELDS:
        if a.get(k) is not None:
            assert np.array_equal(field(b, k), field(a, k), equal_nan=True), k


@pytest.mark.parametrize("aniso", [False, True])
@pytest.mark.parametrize("jacobian", [0, 1])
def test_drop_in_operators_match_reference(aniso, jacobian):
    w = W.aniso(seed=9, ncx=20) if aniso else W.plain_large(seed=9, ncx=22, ncz=18)
    O.shim_sweep(w.model, w.mat, R.FieldSet(w.arrays), 0, aniso, drop_in=False)
    a = R.alloc_operator_fields(w.Nc, w.Nv)
    b = R.alloc_operator_fields(w.Nc, w.Nv)
    assert O.shim_operators(w.model, w.mat, R.FieldSet(clone(w.arrays)), a, jacobian, 1, aniso, drop_in=False) == 0
    assert O.shim_operators(w.model, w.mat, R.FieldSet(clone(w.arrays)), b, jacobian, 1, aniso, drop_in=True) == 0
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k
