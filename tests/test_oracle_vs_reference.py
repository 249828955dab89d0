"""The C restatement (oracle/rheo_oracle.c) against MDOODZ7.0's own sources
compiled by oracle/Makefile: bit-identical on every output.  Skipped where the
reference tree was not available to build oracle/_ref."""
import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from common import clone, field
from golden import cases

pytestmark = pytest.mark.skipif(O.reference() is None, reason="reference not built (oracle/_ref)")

GRIDS = {
    "plain_small_201": (lambda: W.plain_small(seed=0), False, 0),
    "plain_large_96": (lambda: W.plain_large(seed=1, ncx=96), False, 0),
    "plain_large_typical": (lambda: W.plain_large(seed=2, ncx=64, ncz=48, sc=W.TYPICAL), False, 1),
    "plain_large_harmonic": (lambda: W.plain_large(seed=3, ncx=40, eta_average=1), False, 0),
    "plain_large_geometric": (lambda: W.plain_large(seed=4, ncx=50, ncz=30, eta_average=2), False, 0),
    "aniso_64": (lambda: W.aniso(seed=5, ncx=64), True, 0),
    "aniso_typical": (lambda: W.aniso(seed=6, ncx=40, sc=W.TYPICAL), True, 1),
    # edges: one cell, one column, one row, ragged, one phase
    "one_cell": (lambda: W.plain_large(seed=21, ncx=1, ncz=1), False, 0),
    "one_column": (lambda: W.plain_large(seed=22, ncx=1, ncz=9), False, 0),
    "one_row": (lambda: W.plain_large(seed=23, ncx=9, ncz=1), False, 0),
    "ragged_3x300": (lambda: W.plain_large(seed=24, ncx=3, ncz=300), False, 0),
    "one_phase": (lambda: W.plain_large(seed=25, ncx=12, ncz=10, nphases=1), False, 0),
    "aniso_one_row": (lambda: W.aniso(seed=26, ncx=7, ncz=1), True, 0),
}


@pytest.mark.parametrize("name", list(GRIDS))
def test_restatement_bit_identical_on_grids(name):
    builder, aniso, fu = GRIDS[name]
    w = builder()
    a, b = clone(w.arrays), clone(w.arrays)
    O.ref_sweep(w.model, w.mat, R.FieldSet(a), final_update=fu, aniso=aniso)
    rc, _ = O.orc_sweep(w.model, w.mat, R.FieldSet(b), final_update=fu, aniso=aniso)
    assert rc == R.MDZ_OK
    for k in R.VER_INTERP + R.CEN_OUT + R.VER_OUT + ["phase_eta_n", "phase_eta_s"]:
        if k in a:
            assert np.array_equal(field(a, k).view(np.uint64), field(b, k).view(np.uint64)), k


@pytest.mark.parametrize("name", list(cases.POINT_CASES))
@pytest.mark.parametrize("seed", [11, 12])
def test_restatement_bit_identical_on_points(name, seed):
    md, m, pin, aniso, centroid, fu = cases.point_case(name, seed)
    n = pin["phase"].size
    oo, ro = cases.alloc_point_outputs(n), cases.alloc_point_outputs(n)
    pi, po = R.make_points(pin, oo, centroid=centroid, final_update=fu)
    O.orc_points(md, m, pi, po, n, int(aniso))
    if np.any(oo["status"] != 0):  # the reference would exit(): only run it on converging points
        pytest.skip("seed produces a failing point")
    pi, po = R.make_points(pin, ro, centroid=centroid, final_update=fu)
    O.ref_points(md, m, pi, po, n, int(aniso))
    for k in R.PT_OUT:
        assert np.array_equal(oo[k].view(np.uint64), ro[k].view(np.uint64)), k


@pytest.mark.parametrize("where", ["n", "s"])
def test_eta_phys_phase_scale_rebuilds_the_node_values(where):
    """The per-phase eta_phys scale of the parity tests evaluates every phase of a node
    from that node's inputs: its phase average must give back the sweep's eta_phys and
    its eta_VE the sweep's phase_eta."""
    from common import clone, eta_phys_phase_scale
    w = W.plain_large(seed=3, ncx=40)
    c = clone(w.arrays)
    O.orc_sweep(w.model, w.mat, R.FieldSet(c))
    nodes = np.arange(0, 1600, 7)
    scale, eta, eve, perc = eta_phys_phase_scale(w, c, nodes, where, phases=True)
    node = np.sum(np.where(np.abs(perc) > 1e-13, perc * eta, 0.0), axis=1)
    ref = c["eta_phys_" + where][nodes]
    assert np.allclose(node, ref, rtol=1e-14, atol=0)
    pe = np.stack([c["phase_eta_" + where][p][nodes] for p in range(w.mat.Nb_phases)], axis=1)
    act = np.abs(perc) > 1e-13
    assert np.array_equal(eve[act], pe[act])
    assert np.all(scale >= 0.999 * ref)
