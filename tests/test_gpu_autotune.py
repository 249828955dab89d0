"""The launch-shape autotuner: it times every candidate shape on the caller's grid, keeps
the fastest, and changes no result bit (each node is one thread's independent work)."""
import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
from common import clone

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def to_device(arrays):
    return {k: ([torch.from_numpy(x).cuda() for x in v] if isinstance(v, list) else torch.from_numpy(v).cuda())
            for k, v in arrays.items()}


def to_host(d):
    return {k: ([x.cpu().numpy() for x in v] if isinstance(v, list) else v.cpu().numpy()) for k, v in d.items()}


@pytest.mark.parametrize("aniso", [False, True])
def test_autotune_keeps_results_and_picks_a_candidate(aniso):
    w = W.aniso(seed=8, ncx=96) if aniso else W.plain_large(seed=8, ncx=96)
    ctx = R.Context(0)
    try:
        ref = to_device(clone(w.arrays))
        fn = ctx.sweep_aniso if aniso else ctx.sweep
        fn(w.model, w.mat, R.FieldSet(ref), mem=R.MEM_DEVICE)
        assert ctx.launch_shape(aniso) == (128, 0)
        tuned = to_device(clone(w.arrays))
        ms, best, shape = ctx.autotune(w.model, w.mat, R.FieldSet(tuned), aniso=aniso, reps=2)
        print("autotune ms per candidate", np.round(ms, 4), "best", R.Context.AUTOTUNE_CANDIDATES[best], shape)
        assert np.all(ms > 0) and ms[best] == ms.min()
        assert shape[0] == R.Context.AUTOTUNE_CANDIDATES[best][0]
        assert (shape[1] == 0) == (R.Context.AUTOTUNE_CANDIDATES[best][1] == 0)
        # the compacting candidate runs the anisotropic sweep as one thread per node
        want = R.Context.AUTOTUNE_CANDIDATES[best][2]
        assert ctx.launch_form(aniso) == (0 if (aniso and want == 3) else want)
        again = to_device(clone(w.arrays))
        fn(w.model, w.mat, R.FieldSet(again), mem=R.MEM_DEVICE)   # runs with the tuned shape
        a, t, g = to_host(ref), to_host(tuned), to_host(again)
        for k in R.CEN_OUT + R.VER_OUT:
            if a.get(k) is not None:
                assert np.array_equal(a[k], t[k], equal_nan=True), k
                assert np.array_equal(a[k], g[k], equal_nan=True), k
        # the other kind keeps its own shape
        assert ctx.launch_shape(not aniso) == (128, 0)
    finally:
        ctx.close()


@pytest.mark.parametrize("aniso,form", [(False, 1), (True, 1), (False, 2), (True, 2), (False, 3)])
def test_every_form_gives_the_same_bits(aniso, form):
    """The 255-register kernel, the persistent work-counter kernel and the compacting kernel
    against the default one-thread-per-node kernel, bit for bit, from both starts (the
    compacting kernel runs the yielding items' plastic returns in other threads)."""
    w = W.aniso(seed=9, ncx=80) if aniso else W.plain_large(seed=9, ncx=90)
    ctx = R.Context(0)
    try:
        fn = ctx.sweep_aniso if aniso else ctx.sweep
        for flags in (0, R.SWEEP_REF_START):
            ctx.set_launch_shape(aniso, 128, 0, 0)
            ref = to_device(clone(w.arrays))
            fn(w.model, w.mat, R.FieldSet(ref), mem=R.MEM_DEVICE, flags=flags)
            ctx.set_launch_shape(aniso, 128, 0, form)
            assert ctx.launch_form(aniso) == form
            got = to_device(clone(w.arrays))
            _, st = fn(w.model, w.mat, R.FieldSet(got), mem=R.MEM_DEVICE, flags=flags)
            a, g = to_host(ref), to_host(got)
            for k in R.CEN_OUT + R.VER_OUT:
                if a.get(k) is not None:
                    assert np.array_equal(a[k], g[k], equal_nan=True), (flags, k)
            assert st.phase_calls > 0
    finally:
        ctx.close()


def test_compacting_form_rejects_what_it_does_not_run():
    ctx = R.Context(0)
    try:
        assert ctx.lib.mdz_rheo_set_launch_shape(ctx.handle, 1, 128, 0, 3) == R.MDZ_EINVAL  # anisotropic
        assert ctx.lib.mdz_rheo_set_launch_shape(ctx.handle, 0, 64, 0, 3) == R.MDZ_EINVAL   # block 64
    finally:
        ctx.close()


def test_compacting_form_in_banded_host_sweeps_and_with_iterations():
    """Host-memory sweeps in row bands (each band a ranged launch) and the per-item words
    with the compacting form: the same bits as the one-thread-per-node form."""
    w = W.plain_large(seed=10, ncx=120, ncz=300)
    ctx = R.Context(0)
    try:
        out = []
        for form in (0, 3):
            ctx.set_launch_shape(False, 128, 0, form)
            ctx.set_host_bands(7)
            h = clone(w.arrays)
            ctx.sweep(w.model, w.mat, R.FieldSet(h))
            it = clone(w.arrays)
            ctx.sweep(w.model, w.mat, R.FieldSet(it), flags=R.SWEEP_ITERS)
            n = np.zeros(w.mat.Nb_phases * w.Nc, np.int32)
            s = np.zeros(w.mat.Nb_phases * w.Nv, np.int32)
            ctx.get_iterations(n, s)
            out.append((h, n, s))
        (h0, n0, s0), (h3, n3, s3) = out
        for k in R.CEN_OUT + R.VER_OUT:
            if h0.get(k) is not None:
                assert np.array_equal(h0[k], h3[k], equal_nan=True), k
        assert np.array_equal(n0, n3) and np.array_equal(s0, s3)
    finally:
        ctx.close()
