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


# the isotropic inputs the entry point stages from host memory (strain_acc, div, angle and
# the anisotropic ones are not read, so not staged)
STAGED_IN = [k for k in R.PT_IN if k not in ("strain_acc", "div", "angle")]


def staged_bytes(n, n_out):
    """Bytes of the static array a host-memory call with every staged input and n_out
    double outputs (plus iters and status) needs: 256 of statistics, then one slot per
    array rounded up to 256 bytes."""
    r = lambda b: (b + 255) // 256 * 256
    return 256 + r(4 * n) + len(STAGED_IN) * r(8 * n) + n_out * r(8 * n) + 2 * r(4 * n)


def test_oversize_request_is_rejected_untouched():
    n = 1
    while staged_bytes(n, len(R.PT_OUT)) <= R.STATIC_SCRATCH_BYTES:
        n += 64
    fits = n - 64
    while staged_bytes(fits + 1, len(R.PT_OUT)) <= R.STATIC_SCRATCH_BYTES:
        fits += 1
    # the largest request that fits runs, one point more is rejected
    md, m, pin = batch(6, fits, False)
    out = cases.alloc_point_outputs(fits)
    pi, po = R.make_points(pin, out)
    rc, st = R.points_static(md, m, pi, po, fits)
    assert rc == R.MDZ_OK and st.phase_calls == fits
    n = fits + 1
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


def test_calls_allocate_nothing():
    """After the first call on the device, further calls leave the device's free memory
    unchanged: nothing is allocated, not even by a library the call uses."""
    torch = pytest.importorskip("torch")
    md, m, pin = batch(7, 3000, False)
    out = cases.alloc_point_outputs(3000)
    pi, po = R.make_points(pin, out)
    assert R.points_static(md, m, pi, po, 3000)[0] == R.MDZ_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(20):
        assert R.points_static(md, m, pi, po, 3000)[0] == R.MDZ_OK
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_two_threads_on_two_streams_are_serialised():
    """Calls from two host threads, each on its own stream with its own data, give each
    thread the result of the allocating entry point for its data, bit for bit: the calls
    share the one array, and the entry point serialises them."""
    import threading
    torch = pytest.importorskip("torch")
    ctx = R.Context(0)
    try:
        jobs = []
        for seed, n in ((11, 3000), (12, 2200)):
            md, m, pin = batch(seed, n, False)
            ref = cases.alloc_point_outputs(n)
            pi, po = R.make_points(pin, ref)
            assert ctx.points(md, m, pi, po, n) == R.MDZ_OK
            jobs.append((md, m, pin, n, ref))
        streams = [torch.cuda.Stream() for _ in jobs]
        results = [None] * len(jobs)

        def work(k):
            md, m, pin, n, _ = jobs[k]
            got = []
            for _ in range(10):
                out = cases.alloc_point_outputs(n)
                pi, po = R.make_points(pin, out)
                rc, _ = R.points_static(md, m, pi, po, n, stream=streams[k].cuda_stream)
                got.append((rc, out))
            results[k] = got

        threads = [threading.Thread(target=work, args=(k,)) for k in range(len(jobs))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for k, (_, _, _, _, ref) in enumerate(jobs):
            for rc, out in results[k]:
                assert rc == R.MDZ_OK
                for key in list(R.PT_OUT) + ["iters", "status"]:
                    assert np.array_equal(out[key], ref[key], equal_nan=True), (k, key)
    finally:
        ctx.close()
