"""mdz_rheo_points_static (the allocation-free point entry) against mdz_rheo_points.

Both run the same kernel, so the outputs must be identical bit for bit; the static
variant stages through its fixed device array instead of per-call allocations.  Two
calls in a row with different data check that nothing left in the array from the
first call leaks into the second.
"""
import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
from golden import cases

pytestmark = pytest.mark.gpu


def batch(seed, n, aniso):
    rng = np.random.default_rng(seed)
    m = W.materials_plain_large(5)
    if aniso:
        for p in range(5):
            m.gs[p] = 0
    md = W.make_model(8, 8, 5)
    pin = cases._points(rng, n, 5, T=(400.0, 1550.0), aniso=aniso)
    return md, m, pin


def run_both(ctx, md, m, pin, aniso, mem=R.MEM_HOST, to=None):
    n = pin["phase"].size
    ref_out = cases.alloc_point_outputs(n)
    pi, po = R.make_points(pin, ref_out)
    assert ctx.points(md, m, pi, po, n, aniso=int(aniso)) == R.MDZ_OK
    out = cases.alloc_point_outputs(n)
    if to is not None:
        din = {k: to(v) for k, v in pin.items()}
        dout = {k: to(v) for k, v in out.items()}
        pi, po = R.make_points(din, dout)
    else:
        pi, po = R.make_points(pin, out)
    rc, st = R.points_static(md, m, pi, po, n, aniso=int(aniso), mem=mem)
    assert rc == R.MDZ_OK, R.status_string(rc)
    if to is not None:
        out = {k: v.cpu().numpy() for k, v in dout.items()}
    return ref_out, out, st


@pytest.mark.parametrize("aniso", [False, True])
def test_two_calls_in_a_row_match_points(aniso):
    ctx = R.Context(0)
    try:
        for seed, n in ((1, 4000), (2, 2500)):       # the second call is smaller: stale tail in the array
            md, m, pin = batch(seed, n, aniso)
            ref, out, st = run_both(ctx, md, m, pin, aniso)
            for k in list(R.PT_OUT) + ["iters", "status"]:
                assert np.array_equal(out[k], ref[k], equal_nan=True), k
            assert st.phase_calls == n and st.status == R.MDZ_OK and st.kernel_launches == 1
    finally:
        ctx.close()


def test_device_memory_needs_only_the_statistics_block():
    torch = pytest.importorskip("torch")
    ctx = R.Context(0)
    try:
        n = 50_000                                      # far above the host-memory limit
        md, m, pin = batch(3, n, False)
        ref, out, st = run_both(ctx, md, m, pin, False, mem=R.MEM_DEVICE,
                                to=lambda a: torch.from_numpy(a).cuda())
        for k in list(R.PT_OUT) + ["iters", "status"]:
            assert np.array_equal(out[k], ref[k], equal_nan=True), k
        assert st.phase_calls == n
    finally:
        ctx.close()


def test_oversize_request_is_rejected_untouched():
    per_point = 8 * (len(R.PT_IN) + len(R.PT_OUT)) + 4 * 3
    n = R.STATIC_SCRATCH_BYTES // per_point + 100
    md, m, pin = batch(4, n, False)
    out = cases.alloc_point_outputs(n)
    out["eta"][:] = -7.0
    pi, po = R.make_points(pin, out)
    rc, _ = R.points_static(md, m, pi, po, n)
    assert rc == R.MDZ_ESCRATCH
    assert np.all(out["eta"] == -7.0)
    # the same request without most outputs fits
    small = {"eta": np.zeros(n), "status": np.zeros(n, np.int32)}
    pi, po = R.make_points(pin, small)
    rc, st = R.points_static(md, m, pi, po, n)
    assert rc == R.MDZ_OK and st.phase_calls == n and np.all(small["eta"] > 0)


def test_bad_phase_id_is_an_error():
    md, m, pin = batch(5, 300, False)
    pin["phase"][17] = 9
    out = cases.alloc_point_outputs(300)
    pi, po = R.make_points(pin, out)
    rc, _ = R.points_static(md, m, pi, po, 300)
    assert rc == R.MDZ_EINVAL
