"""Many grids in one launch, and sweeps captured as a CUDA graph, against the oracle.

Each grid of a batch has its own size, phase table and time step; after a batched
sweep every grid must match its own oracle sweep at the plain kernel's bar.  The
graph tests perturb the strain rates in each captured sweep (fused into the sweep's
load); the perturbed inputs must equal the host statement of the perturbation exactly,
and the outputs of the last sweep must match the oracle run on those inputs, with the
default start and with the learned warm start.
"""
import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from common import RTOL, clone, worst

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx():
    c = R.Context(0)
    yield c
    c.close()


def to_device(arrays):
    return {k: ([torch.from_numpy(x).cuda() for x in v] if isinstance(v, list) else torch.from_numpy(v).cuda())
            for k, v in arrays.items()}


def to_host(d):
    return {k: ([x.cpu().numpy() for x in v] if isinstance(v, list) else v.cpu().numpy()) for k, v in d.items()}


def check(g, c, w, label):
    errs = worst(g, c, w.arrays, w.model)
    bad = {k: v for k, v in errs.items() if v > RTOL}
    print(label, "max scaled error", max(errs.values()))
    assert not bad, f"{label}: {bad}"


def small_batch(seed=3, n=5):
    return W.many_grids(seed=seed, n=n, lo=9, hi=60)


@pytest.mark.parametrize("flags", [0, R.SWEEP_REF_START])
def test_batch_matches_each_grid(ctx, flags):
    ws = small_batch()
    devs = [to_device(clone(w.arrays)) for w in ws]
    b = R.Batch(ctx, [w.model for w in ws], [w.mat for w in ws], [R.FieldSet(d) for d in devs], flags=flags)
    rc, st = b.sweep()
    assert rc == R.MDZ_OK and st.kernel_launches == 2  # centroid tiles, then vertex tiles
    calls = 0
    for gi, (w, d) in enumerate(zip(ws, devs)):
        c = clone(w.arrays)
        rc2, st2 = O.orc_sweep(w.model, w.mat, R.FieldSet(c))
        assert rc2 == R.MDZ_OK
        calls += st2.phase_calls
        check(to_host(d), c, w, f"grid {gi} ({w.model.Nx - 1} cells, {w.mat.Nb_phases} phases)")
    assert st.phase_calls == calls
    b.close()


def test_batch_matches_single_sweeps_bitwise(ctx):
    ws = small_batch(seed=4, n=4)
    devs = [to_device(clone(w.arrays)) for w in ws]
    b = R.Batch(ctx, [w.model for w in ws], [w.mat for w in ws], [R.FieldSet(d) for d in devs])
    b.sweep()
    for w, d in zip(ws, devs):
        one = to_device(clone(w.arrays))
        ctx.sweep(w.model, w.mat, R.FieldSet(one), mem=R.MEM_DEVICE)
        a, o = to_host(d), to_host(one)
        for k in R.CEN_OUT + R.VER_OUT:
            if a.get(k) is not None:
                assert np.array_equal(a[k], o[k], equal_nan=True), k
    b.close()


def test_captured_graph_with_perturbed_strain_rates(ctx):
    ws = small_batch(seed=5, n=3)
    devs = [to_device(clone(w.arrays)) for w in ws]
    b = R.Batch(ctx, [w.model for w in ws], [w.mat for w in ws], [R.FieldSet(d) for d in devs])
    nsw, amp, seed = 3, 0.05, 11
    b.capture(nsw, amp=amp, seed=seed)
    rc, st = b.launch()
    assert rc == R.MDZ_OK and st.kernel_launches == 2 * nsw  # centroids, vertices; perturbation fused
    total_calls = 0
    for gi, (w, d) in enumerate(zip(ws, devs)):
        h = to_host(d)
        nc = w.Nc
        expect = clone(w.arrays)
        for s in range(nsw):
            for comp, (kc, kv) in enumerate((("exxd", "exxd_s"), ("ezzd", "ezzd_s"), ("exz_n", "exz"))):
                expect[kc] = R.perturb_reference(expect[kc], amp, seed, s, gi, comp, 0)
                expect[kv] = R.perturb_reference(expect[kv], amp, seed, s, gi, comp, nc)
        for k in ("exxd", "ezzd", "exz_n", "exxd_s", "ezzd_s", "exz"):
            assert np.array_equal(h[k], expect[k]), (gi, k)
            assert not np.array_equal(h[k], w.arrays[k])
        rc2, st2 = O.orc_sweep(w.model, w.mat, R.FieldSet(expect))
        total_calls += st2.phase_calls
        check(h, expect, W.Workload(w.name, w.model, w.mat, expect), f"graph grid {gi}")
    assert st.phase_calls == nsw * total_calls
    # a second launch continues the random walk from the perturbed state
    rc, st = b.launch()
    assert rc == R.MDZ_OK
    b.close()


def test_aniso_batch(ctx):
    ws = [W.aniso(seed=40 + i, ncx=n) for i, n in enumerate((17, 31, 24))]
    devs = [to_device(clone(w.arrays)) for w in ws]
    b = R.Batch(ctx, [w.model for w in ws], [w.mat for w in ws], [R.FieldSet(d) for d in devs], aniso=True)
    rc, st = b.sweep()
    assert rc == R.MDZ_OK
    for gi, (w, d) in enumerate(zip(ws, devs)):
        c = clone(w.arrays)
        O.orc_sweep(w.model, w.mat, R.FieldSet(c), aniso=True)
        check(to_host(d), c, w, f"aniso grid {gi}")
    b.close()


@pytest.mark.parametrize("ctas", [1, 7, 456])
def test_persistent_grid_gives_the_same_bits(ctx, ctas):
    """A persistent grid (CTAs striding over the tiles) against one CTA per tile: the same
    node body, so the same bits; a captured graph is dropped by the change."""
    ws = small_batch(seed=12, n=5)
    ref = [to_device(clone(w.arrays)) for w in ws]
    b = R.Batch(ctx, [w.model for w in ws], [w.mat for w in ws], [R.FieldSet(d) for d in ref])
    _, st_ref = b.sweep()
    b.close()
    devs = [to_device(clone(w.arrays)) for w in ws]
    b = R.Batch(ctx, [w.model for w in ws], [w.mat for w in ws], [R.FieldSet(d) for d in devs])
    b.capture(2)
    b.set_grid(ctas)
    rc, _ = b.launch(check=False)
    assert rc == R.MDZ_ENOTREADY
    rc, st = b.sweep()
    assert rc == R.MDZ_OK and st.kernel_launches == 2
    assert (st.phase_calls, st.newton_iters, st.plastic_calls) == (st_ref.phase_calls, st_ref.newton_iters,
                                                                   st_ref.plastic_calls)
    for d, r in zip(devs, ref):
        a, o = to_host(d), to_host(r)
        for k in R.CEN_OUT + R.VER_OUT:
            if a.get(k) is not None:
                assert np.array_equal(a[k], o[k], equal_nan=True), k
    b.set_grid(0)
    b.close()


def expected_inputs(w, gi, nsw, amp, seed):
    """The host statement of `nsw` perturbations of grid gi's strain rates."""
    expect = clone(w.arrays)
    for s in range(nsw):
        for comp, (kc, kv) in enumerate((("exxd", "exxd_s"), ("ezzd", "ezzd_s"), ("exz_n", "exz"))):
            expect[kc] = R.perturb_reference(expect[kc], amp, seed, s, gi, comp, 0)
            expect[kv] = R.perturb_reference(expect[kv], amp, seed, s, gi, comp, w.Nc)
    return expect


@pytest.fixture(scope="module")
def network(ctx):
    import mdz_warmstart as WS
    X, Y = WS.collect(ctx, [W.plain_large(seed=150, ncx=129), W.plain_small(seed=151, ncx=129)])
    w, _, _ = WS.train(ctx, X, Y, WS.FEAT_ISO, WS.default_cfg(epochs=3, batch=4096))
    return w


def test_warm_batch_matches_warm_single_sweeps_bitwise(ctx, network):
    ctx.set_warmstart(network, R.DEFAULT_START)
    ws = small_batch(seed=8, n=4)
    devs = [to_device(clone(w.arrays)) for w in ws]
    b = R.Batch(ctx, [w.model for w in ws], [w.mat for w in ws], [R.FieldSet(d) for d in devs],
                flags=R.SWEEP_WARMSTART)
    rc, st = b.sweep()
    assert rc == R.MDZ_OK and st.kernel_launches == 2
    for w, d in zip(ws, devs):
        one = to_device(clone(w.arrays))
        ctx.sweep(w.model, w.mat, R.FieldSet(one), mem=R.MEM_DEVICE, flags=R.SWEEP_WARMSTART)
        a, o = to_host(d), to_host(one)
        for k in R.CEN_OUT + R.VER_OUT:
            if a.get(k) is not None:
                assert np.array_equal(a[k], o[k], equal_nan=True), k
    b.close()


def test_warm_graph_of_20_perturbed_sweeps(ctx, network):
    """The many-grid form on a few grids: one batch of uneven grids with the learned warm start,
    20 sweeps captured as one graph, strain rates perturbed by +-5 % in each."""
    ctx.set_warmstart(network, R.DEFAULT_START)
    ws = small_batch(seed=9, n=4)
    devs = [to_device(clone(w.arrays)) for w in ws]
    b = R.Batch(ctx, [w.model for w in ws], [w.mat for w in ws], [R.FieldSet(d) for d in devs],
                flags=R.SWEEP_WARMSTART)
    nsw, amp, seed = 20, 0.05, 2026
    b.capture(nsw, amp=amp, seed=seed)
    rc, st = b.launch()
    assert rc == R.MDZ_OK and st.kernel_launches == 2 * nsw and st.mma_fault == 0
    calls = 0
    for gi, (w, d) in enumerate(zip(ws, devs)):
        h = to_host(d)
        expect = expected_inputs(w, gi, nsw, amp, seed)
        for k in ("exxd", "ezzd", "exz_n", "exxd_s", "ezzd_s", "exz"):
            assert np.array_equal(h[k], expect[k]), (gi, k)
        rc2, st2 = O.orc_sweep(w.model, w.mat, R.FieldSet(expect))
        assert rc2 == R.MDZ_OK
        calls += st2.phase_calls
        check(h, expect, W.Workload(w.name, w.model, w.mat, expect), f"warm graph grid {gi}")
    assert st.phase_calls == nsw * calls
    assert st.newton_iters <= 1.05 * st.phase_calls  # about one FP64 evaluation per local solve
    b.close()


def test_batch_argument_checks(ctx):
    ws = small_batch(seed=6, n=2)
    devs = [to_device(clone(w.arrays)) for w in ws]
    ctx.set_warmstart(None)
    with pytest.raises(R.RheoError):  # no network installed
        R.Batch(ctx, [w.model for w in ws], [w.mat for w in ws], [R.FieldSet(d) for d in devs],
                flags=R.SWEEP_WARMSTART)
    with pytest.raises(R.RheoError):
        R.Batch(ctx, [w.model for w in ws], [w.mat for w in ws], [R.FieldSet(d) for d in devs],
                flags=R.SWEEP_WARMSTART | R.SWEEP_REF_START)
    b = R.Batch(ctx, [w.model for w in ws], [w.mat for w in ws], [R.FieldSet(d) for d in devs])
    rc, _ = b.launch(check=False)
    assert rc == R.MDZ_ENOTREADY
    b.close()
