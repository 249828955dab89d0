"""The oracle against the golden fixtures produced by MDOODZ7.0's own code
(tests/golden/make_golden.py): bit-identical outputs, and unchanged inputs."""
import os

import numpy as np
import pytest

import mdz_rheo as R
import oracle_lib as O
from golden import cases
from golden.make_golden import grid_inputs_digest, grid_outputs, point_inputs_digest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", list(cases.GRID_CASES))
def test_oracle_grid_matches_golden(name):
    builder, aniso, fu = cases.GRID_CASES[name]
    w = builder()
    g = np.load(os.path.join(GOLDEN, f"grid_{name}.npz"))
    assert str(g["inputs_sha256"]) == grid_inputs_digest(w), "input generator changed"
    rc, st = O.orc_sweep(w.model, w.mat, R.FieldSet(w.arrays), final_update=fu, aniso=aniso)
    assert rc == R.MDZ_OK
    out = grid_outputs(w.arrays)
    for k, v in out.items():
        assert np.array_equal(v.view(np.uint64), g[k].view(np.uint64)), k


@pytest.mark.parametrize("name", list(cases.POINT_CASES))
def test_oracle_points_match_golden(name):
    md, m, pin, aniso, centroid, fu = cases.point_case(name)
    g = np.load(os.path.join(GOLDEN, f"points_{name}.npz"))
    assert str(g["inputs_sha256"]) == point_inputs_digest(pin), "input generator changed"
    n = pin["phase"].size
    out = cases.alloc_point_outputs(n)
    pi, po = R.make_points(pin, out, centroid=centroid, final_update=fu)
    assert O.orc_points(md, m, pi, po, n, int(aniso)) == R.MDZ_OK
    for k in R.PT_OUT:
        assert np.array_equal(out[k].view(np.uint64), g[k].view(np.uint64)), k


def swept_grid(grid_case):
    """The inputs of a grid case with the reference sweep's outputs (from its golden
    fixture) filled in: the state RheologicalOperators reads."""
    builder, aniso, fu = cases.GRID_CASES[grid_case]
    w = builder()
    g = np.load(os.path.join(GOLDEN, f"grid_{grid_case}.npz"))
    for k in g.files:
        if k == "inputs_sha256":
            continue
        if k in ("phase_eta_n", "phase_eta_s"):
            for p in range(w.mat.Nb_phases):
                w.arrays[k][p][:] = g[k][p]
        elif w.arrays.get(k) is not None:
            w.arrays[k][:] = g[k]
    return w, aniso


@pytest.mark.parametrize("name", list(cases.OPERATOR_CASES))
def test_oracle_operators_match_golden(name):
    grid_case, jac, comp = cases.OPERATOR_CASES[name]
    w, aniso = swept_grid(grid_case)
    g = np.load(os.path.join(GOLDEN, f"operators_{name}.npz"))
    assert str(g["inputs_sha256"]) == grid_inputs_digest(cases.GRID_CASES[grid_case][0]()), "input generator changed"
    ops = R.alloc_operator_fields(w.Nc, w.Nv)
    assert O.orc_operators(w.model, w.mat, R.FieldSet(w.arrays), ops, jac, comp, aniso) == R.MDZ_OK
    for k in R.OPS_N + R.OPS_S:
        assert np.array_equal(ops[k].view(np.uint64), g[k].view(np.uint64)), k
