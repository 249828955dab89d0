"""RheologicalOperators (Picard and Newton, with the finite-difference derivatives of
FD_Jacobian.c): the C restatement against the reference compiled from its own sources,
bit for bit, after a sweep has updated the grid."""
import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from common import clone

pytestmark = pytest.mark.skipif(O.reference() is None, reason="reference build absent (oracle/_ref)")


def dilatant(w):
    """Dilation 10 deg and a finite bulk modulus, so the plastic-divergence terms matter."""
    for k in ("dil_n", "dil_s"):
        w.arrays[k][:] = 10.0 * W.DEG
    for k in ("bet_n", "bet_s"):
        w.arrays[k][:] = 1e-11
    return w


def with_density(w):
    for p in range(w.mat.Nb_phases):
        w.mat.density_model[p] = 1
        w.mat.rho[p], w.mat.alp[p], w.mat.bet[p] = 3300.0, 3e-5, 1e-11
    return w


CASES = {
    "iso": (lambda: W.plain_large(seed=3, ncx=40, ncz=30), False),
    "iso_harmonic": (lambda: W.plain_large(seed=4, ncx=31, eta_average=1), False),
    "iso_geometric": (lambda: W.plain_large(seed=5, ncx=33, ncz=28, eta_average=2), False),
    "iso_typical_scale": (lambda: W.plain_large(seed=6, ncx=30, sc=W.TYPICAL), False),
    "iso_dilatant_density": (lambda: with_density(dilatant(W.plain_large(seed=7, ncx=36))), False),
    "aniso": (lambda: W.aniso(seed=5, ncx=30), True),
    "aniso_dilatant": (lambda: dilatant(W.aniso(seed=8, ncx=26)), True),
}


@pytest.mark.parametrize("jacobian", [0, 1])
@pytest.mark.parametrize("compressible", [0, 1])
@pytest.mark.parametrize("name", list(CASES))
def test_operators_restatement_is_the_reference(name, jacobian, compressible):
    make, aniso = CASES[name]
    w = make()
    rc = O.ref_sweep(w.model, w.mat, R.FieldSet(w.arrays), 0, aniso)
    assert rc == 0
    a = R.alloc_operator_fields(w.Nc, w.Nv)
    b = R.alloc_operator_fields(w.Nc, w.Nv)
    assert O.ref_operators(w.model, w.mat, R.FieldSet(clone(w.arrays)), a, jacobian, compressible, aniso) == 0
    assert O.orc_operators(w.model, w.mat, R.FieldSet(clone(w.arrays)), b, jacobian, compressible, aniso) == 0
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k
    if jacobian:
        assert np.any(a["D14_n"] != 0.0) and np.any(a["D34_s"] != 0.0)
