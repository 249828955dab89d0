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
        assert ctx.launch_form(aniso) == R.Context.AUTOTUNE_CANDIDATES[best][2]
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


@pytest.mark.parametrize("aniso", [False, True])
@pytest.mark.parametrize("form", [1, 2])
def test_every_form_gives_the_same_bits(aniso, form):
    """The 255-register kernel and the persistent work-counter kernel against the default
    one-thread-per-node kernel, bit for bit, from both starts."""
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
