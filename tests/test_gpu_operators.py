"""RheologicalOperators on the GPU against the reference (golden fixtures) and the oracle.

The Picard operator is a few products per node and matches to rounding.  The Newton
operator contains central differences of perturbed local solves with steps of 1e-5
(centroids) and 1e-7 (vertices) of the strain rate and pressure.  Each local solve is
defined by the reference only to its stopping test |r| < 1e-13 Eii, so a difference
quotient carries up to about 1e-13 / 1e-5 = 1e-8 (centroids) and 1e-13 / 1e-7 = 1e-6
(vertices) of the viscosity as noise in the reference itself.  A local solve may stop
anywhere below the threshold and its terms carry the exponents (n up to ~5), so the bars
take delta = 1e-12: delta / (2 x 1e-5) = 5e-8 at centroids and delta / (2 x 1e-7) = 5e-6
at vertices.  Each coefficient is measured against its natural magnitude: 2 eta for the
viscous coefficients; 2 eta Eii / |P| for the pressure columns D14, D24, D34 (the size
they have when eta changes by order one over the pressure); rho / |P| for d(rho)/dP.
"""
import os

import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from common import clone, node_Eii
from golden import cases
from test_golden import GOLDEN, swept_grid

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

VISCOUS_N = ["D11_n", "D12_n", "D13_n", "D21_n", "D22_n", "D23_n"]
VISCOUS_S = ["D31_s", "D32_s", "D33_s"]
PRESSURE = ["D14_n", "D24_n", "D34_s", "drhodp_n"]
BAR_N, BAR_S = 5e-8, 5e-6


@pytest.fixture(scope="module")
def ctx():
    c = R.Context(0)
    yield c
    c.close()


def op_errors(got, ref, arrays, model, mat):
    out = {}
    with np.errstate(divide="ignore", invalid="ignore"):
        p_n, p_s = np.abs(arrays["p_in"]), np.abs(arrays["P_s"])
        natural = {"D14_n": 2.0 * np.abs(arrays["eta_n"]) * node_Eii(arrays, model, "n") / p_n,
                   "D34_s": 2.0 * np.abs(arrays["eta_s"]) * node_Eii(arrays, model, "s") / p_s,
                   "drhodp_n": max(mat.rho[p] for p in range(mat.Nb_phases)) / p_n}
    natural["D24_n"] = natural["D14_n"]
    for k in VISCOUS_N + VISCOUS_S + PRESSURE:
        g, r = np.asarray(got[k], np.float64), np.asarray(ref[k], np.float64)
        if k in VISCOUS_N:
            scale = np.maximum(np.abs(r), 2.0 * np.abs(arrays["eta_n"]))
        elif k in VISCOUS_S:
            scale = np.maximum(np.abs(r), 2.0 * np.abs(arrays["eta_s"]))
        else:
            scale = np.maximum(np.abs(r), np.nan_to_num(natural[k], nan=np.inf))
        scale = np.where(scale > 0, scale, 1.0)
        e = np.where(g == r, 0.0, np.abs(g - r) / scale)
        out[k] = float(np.max(e)) if e.size else 0.0
        if e.size and out[k] > 0:
            i = int(np.argmax(e))
            WORST[k] = (i, float(g[i]), float(r[i]), float(scale[i]))
    return out


WORST = {}


def check(errs, label, jac):
    bad = {k: v for k, v in errs.items() if v > (BAR_S if k.endswith("_s") else BAR_N) * (1 if jac else 1e-4)}
    print(label, {k: f"{v:.1e}" for k, v in errs.items()})
    for k in bad:
        print("  worst", k, "(node, gpu, reference, scale) =", WORST.get(k))
    assert not bad, f"{label}: {bad}"


@pytest.mark.parametrize("flags", [R.SWEEP_REF_START, 0])
@pytest.mark.parametrize("name", list(cases.OPERATOR_CASES))
def test_gpu_operators_match_golden(ctx, name, flags):
    grid_case, jac, comp = cases.OPERATOR_CASES[name]
    w, aniso = swept_grid(grid_case)
    g = np.load(os.path.join(GOLDEN, f"operators_{name}.npz"))
    ops = R.alloc_operator_fields(w.Nc, w.Nv)
    rc, st = ctx.operators(w.model, w.mat, R.FieldSet(w.arrays), ops, jacobian=jac, compressible=comp,
                           aniso=aniso, flags=flags)
    assert rc == R.MDZ_OK
    if jac:
        assert st.phase_calls > 0
    check(op_errors(ops, {k: g[k] for k in g.files if k != "inputs_sha256"}, w.arrays, w.model, w.mat),
          f"{name} flags={flags}", jac)


@pytest.mark.parametrize("aniso", [False, True])
def test_gpu_operators_after_gpu_sweep_match_oracle(ctx, aniso):
    w = W.aniso(seed=21, ncx=64, ncz=48) if aniso else W.plain_large(seed=21, ncx=64, ncz=48)
    d = {k: ([torch.from_numpy(x).cuda() for x in v] if isinstance(v, list) else torch.from_numpy(v).cuda())
         for k, v in w.arrays.items()}
    fn = ctx.sweep_aniso if aniso else ctx.sweep
    fn(w.model, w.mat, R.FieldSet(d), mem=R.MEM_DEVICE)
    ops_d = R.alloc_operator_fields(w.Nc, w.Nv, like=d["eta_n"])
    rc, st = ctx.operators(w.model, w.mat, R.FieldSet(d), ops_d, jacobian=1, aniso=aniso, mem=R.MEM_DEVICE,
                           flags=R.SWEEP_REF_START)
    assert rc == R.MDZ_OK
    host = {k: ([x.cpu().numpy() for x in v] if isinstance(v, list) else v.cpu().numpy()) for k, v in d.items()}
    ops_c = R.alloc_operator_fields(w.Nc, w.Nv)
    assert O.orc_operators(w.model, w.mat, R.FieldSet(clone(host)), ops_c, 1, 0, aniso) == R.MDZ_OK
    got = {k: v.cpu().numpy() for k, v in ops_d.items()}
    check(op_errors(got, ops_c, host, w.model, w.mat), f"gpu sweep + operators, aniso={aniso}", 1)


def test_gpu_picard_matches_oracle_exactly(ctx):
    w = W.plain_large(seed=22, ncx=40, ncz=40)
    ctx.sweep(w.model, w.mat, R.FieldSet(w.arrays))
    a = R.alloc_operator_fields(w.Nc, w.Nv)
    b = R.alloc_operator_fields(w.Nc, w.Nv)
    ctx.operators(w.model, w.mat, R.FieldSet(w.arrays), a, jacobian=0)
    O.orc_operators(w.model, w.mat, R.FieldSet(clone(w.arrays)), b, 0, 0, False)
    for k in R.OPS_N + R.OPS_S:
        assert np.array_equal(a[k], b[k]), k


def _newton_both_forms(ctx, w, aniso=False, comp=0, flags=0):
    out = []
    for form in (0, R.OPS_PER_NODE):  # plastic returns compacted per CTA (the default), one thread per node
        ops = R.alloc_operator_fields(w.Nc, w.Nv)
        for k in ops:  # the Newton operator leaves drhodp_n at air cells untouched
            ops[k][:] = 7.0
        rc, st = ctx.operators(w.model, w.mat, R.FieldSet(clone(w.arrays)), ops, jacobian=1, compressible=comp,
                               aniso=aniso, flags=flags | form)
        assert rc == R.MDZ_OK
        out.append((ops, st.phase_calls))
    return out


@pytest.mark.parametrize("flags", [0, R.SWEEP_REF_START])
@pytest.mark.parametrize("name", [n for n, c in cases.OPERATOR_CASES.items() if c[1] == 1])
def test_gpu_compacting_newton_operator_is_bitwise_one_thread_per_node(ctx, name, flags):
    """The isotropic Newton operator runs its Drucker-Prager returns packed into the first
    warps of each CTA; the result must be the one-thread-per-node operator's, bit for bit
    (the anisotropic operator keeps one thread per node in both forms)."""
    grid_case, _, comp = cases.OPERATOR_CASES[name]
    w, aniso = swept_grid(grid_case)
    (a, ca), (b, cb) = _newton_both_forms(ctx, w, aniso, comp, flags)
    assert ca == cb > 0
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), (name, k)


def test_gpu_compacting_newton_operator_ragged_grid(ctx):
    """A grid whose node count leaves the last CTA partly empty, with many yielding items."""
    w = W.plain_large(seed=23, ncx=97, ncz=75)
    ctx.sweep(w.model, w.mat, R.FieldSet(w.arrays))
    assert (w.Nc + w.Nv) % 128 != 0
    (a, ca), (b, cb) = _newton_both_forms(ctx, w)
    assert ca == cb > 0
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k
