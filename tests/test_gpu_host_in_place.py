"""Host arrays used in place by the entry points other than the sweep.

RheologicalOperators, StrainRateComponents, the input preparation (softening, shear
modulus), UpdateParticleStress and P2Mastah read and write host arrays that the device can address directly, without device
copies: page-locked arrays mapped at the same pointer, and pageable arrays where the GPU
reads pageable memory through the host page tables (Grace-Blackwell).  Any other array, or
MDZ_SWEEP_STAGED, goes through the context's device mirrors.  Each case checks that the
three forms (page-locked, staged by the flag, pageable) give the same bits and the same
byte counts, and that an in-place call allocates no mirrors (free device memory of a fresh
context) while a staged one does.
"""
import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
from common import clone

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

MiB = 1 << 20


def pinned(d):
    return {k: (None if v is None else [torch.from_numpy(np.array(x, copy=True)).pin_memory() for x in v]
                if isinstance(v, list) else torch.from_numpy(np.array(v, copy=True)).pin_memory())
            for k, v in d.items()}


def as_numpy(d):
    return {k: (None if v is None else [x.numpy() if hasattr(x, "numpy") else x for x in v]
                if isinstance(v, list) else (v.numpy() if hasattr(v, "numpy") else v)) for k, v in d.items()}


def free_bytes():
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info(0)[0]


def three_ways(call, arrays):
    """(page-locked, staged by the flag, pageable): outputs, statistics, device bytes the
    call took in a fresh context, and whether pageable arrays are used in place."""
    out = []
    pageable_in_place = None
    for form in ("in_place", "flag", "pageable"):
        a = pinned(arrays) if form != "pageable" else clone(arrays)
        ctx = R.Context(0)
        pageable_in_place = ctx.pageable_in_place()
        f0 = free_bytes()
        rc, st = call(ctx, a, R.SWEEP_STAGED if form == "flag" else 0)
        used = f0 - free_bytes()
        ctx.close()
        assert rc == R.MDZ_OK, form
        out.append((as_numpy(a), st, used))
    return out, pageable_in_place


def check_same(result, keys, rtol=None):
    """Outputs bit for bit (or within rtol of the largest value, for sums that FP64 atomics
    add in another order on every run), byte counts equal, and device memory: the in-place
    call allocates no mirrors (scratch only), a staged one a mirror per array (tens of MiB)."""
    res, pageable_in_place = result
    (a, sa, ua), (b, sb, ub), (c, sc, uc) = res
    for k in keys:
        if a.get(k) is None:
            continue
        x, y, z = (np.concatenate(v) if isinstance(v, list) else v for v in (a[k], b[k], c[k]))
        if rtol is None:
            assert np.array_equal(x, y, equal_nan=True) and np.array_equal(x, z, equal_nan=True), k
        else:
            scale = max(float(np.max(np.abs(x))), 1e-300)
            assert float(np.max(np.abs(x - y))) <= rtol * scale and float(np.max(np.abs(x - z))) <= rtol * scale, k
    assert (sa.h2d_bytes, sa.d2h_bytes) == (sb.h2d_bytes, sb.d2h_bytes) == (sc.h2d_bytes, sc.d2h_bytes)
    assert sa.h2d_bytes > 0 and sa.d2h_bytes > 0
    assert ub - ua >= 24 * MiB, (ua, ub)
    if pageable_in_place:  # the GPU reads pageable memory through the host page tables
        assert abs(uc - ua) <= 8 * MiB, (ua, uc)
    else:
        assert uc - ua >= 24 * MiB, (ua, uc)


@pytest.mark.parametrize("jac", [0, 1])
def test_operators_in_place(jac):
    big = W.plain_large(seed=5, ncx=400, ncz=360)
    c = R.Context(0)
    c.sweep(big.model, big.mat, R.FieldSet(big.arrays))  # the state the operator linearises
    c.close()
    arrays = dict(big.arrays)
    ops = R.alloc_operator_fields(big.Nc, big.Nv)
    for k in ops:
        ops[k][:] = 3.0
    arrays.update({"op_" + k: v for k, v in ops.items()})

    def call(ctx, a, flags):
        fields = {k: v for k, v in a.items() if not k.startswith("op_")}
        o = {k[3:]: v for k, v in a.items() if k.startswith("op_")}
        return ctx.operators(big.model, big.mat, R.FieldSet(fields), o, jacobian=jac, flags=flags)

    res = three_ways(call, arrays)
    check_same(res, ["op_" + k for k in R.OPS_N + R.OPS_S])


def test_strain_rates_in_place():
    w = W.velocity_field(seed=8, ncx=700, ncz=650, air=0.2, periodic=1)
    res = three_ways(lambda ctx, a, flags: ctx.strain_rates(w.model, w.info["dx"], w.info["dz"], a,
                                                             out_of_plane=1, compressible=1.0, flags=flags),
                     w.arrays)
    check_same(res, R.SR_N + R.SR_S)


@pytest.mark.parametrize("step", ["softening", "shear_modulus"])
def test_input_preparation_in_place(step):
    w = W.prep_workload(seed=9, ncx=700, ncz=650, nphases=4, air=0.1, periodic=1)

    def call(ctx, a, flags):
        if step == "softening":
            return ctx.softening(w.model, w.mat, R.PrepFieldSet(a), 1, 0, 1, flags=flags)
        return ctx.shear_modulus(w.model, w.mat, R.PrepFieldSet(a), flags=flags)

    res = three_ways(call, w.arrays)
    check_same(res, [k for k in w.arrays if k not in ("phase_perc_n", "phase_perc_s", "BCp_type", "BCg_type")])


def marker_case():
    w = W.marker_workload(seed=31, ncx=300, ncz=280, markers_per_cell=16, air=0.2, periodic=1)
    arrays = {"g_" + k: v for k, v in w.arrays.items()}
    arrays.update({"m_" + k: v for k, v in w.info["markers"].items()})
    return w, arrays


def split(a):
    return ({k[2:]: v for k, v in a.items() if k.startswith("g_")},
            {k[2:]: v for k, v in a.items() if k.startswith("m_")})


@pytest.mark.parametrize("stencil,rot,sub", [(1, 1, 0), (9, 2, 0), (1, 1, 2)])
def test_marker_stress_in_place(stencil, rot, sub):
    from golden.make_golden import marker_opts
    w, arrays = marker_case()
    opts = marker_opts(1, rot, 1, 1, stencil, sub, G=w.info["G"])

    def call(ctx, a, flags):
        g, m = split(a)
        return ctx.marker_stress(w.model, opts, g, m, w.info["dx"], w.info["dz"], flags=flags)

    res = three_ways(call, arrays)
    check_same(res, ["m_sxxd", "m_szzd", "m_sxz", "m_nx", "m_nz", "g_wxz"], rtol=1e-12 if sub == 2 else None)


@pytest.mark.parametrize("stencil", [1, 9])
def test_p2mastah_in_place(stencil):
    w, arrays = marker_case()
    rng = np.random.default_rng(3)
    arrays["values"] = rng.random(w.info["markers"]["x"].size)
    arrays["node_n"] = np.zeros((w.model.Nx - 1) * (w.model.Nz - 1))
    arrays["node_s"] = np.zeros(w.model.Nx * w.model.Nz)

    def call(ctx, a, flags):
        g, m = split(a)
        return ctx.p2mastah(w.model, g, m, a["values"], 0, stencil, a["node_n"], a["node_s"], w.info["dx"],
                            w.info["dz"], flags=flags)

    res = three_ways(call, arrays)
    check_same(res, ["node_n", "node_s"], rtol=1e-12)

