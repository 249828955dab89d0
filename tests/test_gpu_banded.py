"""Sweeps of host arrays staged in row bands (copies overlapping the kernels) against the
one-shot host sweep and the device-resident sweep: every output bit for bit, for any
band count, with periodic x, air rows and uneven band edges; and host arrays that the
kernels read and write in place.  MDZ_SWEEP_STAGED makes the banded path run where the GPU
could address the arrays directly."""
import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
from common import clone

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx():
    c = R.Context(0)
    yield c
    c.set_host_bands(0)
    c.close()


def with_air_and_periodic(w, air_rows=9):
    """Air above the top `air_rows` rows (BCp 31, BCg 30) and periodic x."""
    m, a = w.model, w.arrays
    a["BCp_type"].reshape(m.Nz - 1, m.Nx - 1)[-air_rows:, :] = 31
    a["BCg_type"].reshape(m.Nz, m.Nx)[-air_rows:, :] = 30
    m.periodic_x = 1
    return w


CASES = {
    "plain_large_96x257": (lambda: W.plain_large(seed=21, ncx=96, ncz=257), False),
    "plain_large_air_periodic": (lambda: with_air_and_periodic(W.plain_large(seed=22, ncx=70, ncz=131)), False),
    "aniso_80x150_air_periodic": (lambda: with_air_and_periodic(W.aniso(seed=23, ncx=80, ncz=150)), True),
}


def same(a, b):
    for k in a:
        x, y = a[k], b[k]
        if isinstance(x, list):
            for i, (u, v) in enumerate(zip(x, y)):
                assert np.array_equal(np.asarray(u).view(np.uint8), np.asarray(v).view(np.uint8)), (k, i)
        else:
            assert np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8)), k


@pytest.mark.parametrize("name", list(CASES))
def test_banded_host_sweep_is_the_one_shot_sweep(ctx, name):
    make, aniso = CASES[name]
    w = make()
    fn = ctx.sweep_aniso if aniso else ctx.sweep
    ctx.set_host_bands(1)
    one = clone(w.arrays)
    _, st1 = fn(w.model, w.mat, R.FieldSet(one), flags=R.SWEEP_STAGED)
    assert st1.kernel_launches == 2  # the centroid kernel and the vertex kernel
    # the device-resident sweep on the same inputs
    dev = {k: ([torch.from_numpy(x.copy()).cuda() for x in v] if isinstance(v, list) else
               torch.from_numpy(v.copy()).cuda()) for k, v in w.arrays.items()}
    fn(w.model, w.mat, R.FieldSet(dev), mem=R.MEM_DEVICE)
    same(one, {k: ([x.cpu().numpy() for x in v] if isinstance(v, list) else v.cpu().numpy()) for k, v in dev.items()})
    for bands in (2, 3, 7, 16):
        ctx.set_host_bands(bands)
        got = clone(w.arrays)
        _, st = fn(w.model, w.mat, R.FieldSet(got), flags=R.SWEEP_STAGED)
        # a vertex kernel per band and a centroid kernel per band with centroid rows (all but
        # a last band holding only the last vertex row)
        assert 2 * min(bands, w.model.Nz) - 1 <= st.kernel_launches <= 2 * min(bands, w.model.Nz)
        assert st.phase_calls == st1.phase_calls and st.newton_iters == st1.newton_iters
        assert st.h2d_bytes == st1.h2d_bytes and st.d2h_bytes == st1.d2h_bytes
        same(one, got)
    ctx.set_host_bands(0)


def test_banded_sweep_reports_the_failing_node(ctx):
    """A node whose local solve fails in a later band: the same status and node as the
    one-shot sweep."""
    w = W.plain_large(seed=24, ncx=40, ncz=200)
    c1 = w.model.Nx * 150 + 7  # a vertex in the fourth of five bands
    w.arrays["exz"][c1] = np.nan
    ctx.set_host_bands(1)
    rc1, st1 = ctx.sweep(w.model, w.mat, R.FieldSet(clone(w.arrays)), flags=R.SWEEP_STAGED, check=False)
    ctx.set_host_bands(5)
    rc5, st5 = ctx.sweep(w.model, w.mat, R.FieldSet(clone(w.arrays)), flags=R.SWEEP_STAGED, check=False)
    ctx.set_host_bands(0)
    assert rc1 == rc5 and st1.status == st5.status and st1.error_node == st5.error_node


def test_host_bands_argument_checked(ctx):
    with pytest.raises(R.RheoError):
        ctx.set_host_bands(17)
    with pytest.raises(R.RheoError):
        ctx.set_host_bands(-1)


def pinned(arrays):
    return {k: ([torch.from_numpy(x.copy()).pin_memory() for x in v] if isinstance(v, list)
                else torch.from_numpy(v.copy()).pin_memory()) for k, v in arrays.items()}


def host_view(d):
    return {k: ([x.numpy() for x in v] if isinstance(v, list) else v.numpy()) for k, v in d.items()}


@pytest.mark.parametrize("aniso", [False, True])
def test_direct_sweep_of_page_locked_host_arrays(ctx, aniso):
    """Page-locked host arrays are read and written by the kernels in place (no staging
    copies: two launches, no bands), with the same bits and the same host<->device byte
    counts as the staged sweep in row bands (MDZ_SWEEP_STAGED) and as the sweep of
    device-resident copies."""
    w = W.aniso(seed=41, ncx=300, ncz=280) if aniso else with_air_and_periodic(W.plain_large(seed=41, ncx=300, ncz=280))
    fn = ctx.sweep_aniso if aniso else ctx.sweep
    ctx.set_host_bands(0)
    direct = pinned(clone(w.arrays))
    rc, st_d = fn(w.model, w.mat, R.FieldSet(direct))
    assert rc == R.MDZ_OK and st_d.kernel_launches == 2
    staged = pinned(clone(w.arrays))
    rc, st_s = fn(w.model, w.mat, R.FieldSet(staged), flags=R.SWEEP_STAGED)
    assert rc == R.MDZ_OK and st_s.kernel_launches > 2  # row bands
    dev = {k: ([torch.from_numpy(x.copy()).cuda() for x in v] if isinstance(v, list)
               else torch.from_numpy(v.copy()).cuda()) for k, v in w.arrays.items()}
    fn(w.model, w.mat, R.FieldSet(dev), mem=R.MEM_DEVICE)
    torch.cuda.synchronize()
    a, b = host_view(direct), host_view(staged)
    c = {k: ([x.cpu().numpy() for x in v] if isinstance(v, list) else v.cpu().numpy()) for k, v in dev.items()}
    for k in R.VER_INTERP + R.CEN_OUT + R.VER_OUT + ["phase_eta_n", "phase_eta_s"]:
        if a.get(k) is None:
            continue
        x, y, z = (np.concatenate(v) if isinstance(v, list) else v for v in (a[k], b[k], c[k]))
        assert np.array_equal(x, y, equal_nan=True) and np.array_equal(x, z, equal_nan=True), k
    assert (st_d.h2d_bytes, st_d.d2h_bytes) == (st_s.h2d_bytes, st_s.d2h_bytes)
    assert st_d.phase_calls == st_s.phase_calls


def test_pageable_arrays(ctx):
    """One pageable array among page-locked ones, and all arrays pageable: in place where the
    GPU reads pageable memory through the host page tables (two launches), else the sweep
    stages everything (bands); the same bits as the staged sweep either way."""
    w = W.plain_large(seed=42, ncx=200, ncz=260)
    ctx.set_host_bands(0)
    in_place = ctx.pageable_in_place()
    ref = clone(w.arrays)
    rc, st = ctx.sweep(w.model, w.mat, R.FieldSet(ref), flags=R.SWEEP_STAGED)
    assert rc == R.MDZ_OK and st.kernel_launches > 2
    mixed = pinned(clone(w.arrays))
    mixed["T"] = torch.from_numpy(w.arrays["T"].copy())  # pageable
    plain = clone(w.arrays)  # numpy: pageable
    for arrays in (mixed, plain):
        rc, st = ctx.sweep(w.model, w.mat, R.FieldSet(arrays))
        assert rc == R.MDZ_OK
        assert (st.kernel_launches == 2) if in_place else (st.kernel_launches > 2)
        got = host_view(arrays) if arrays is mixed else arrays
        for k in R.VER_INTERP + R.CEN_OUT + R.VER_OUT + ["phase_eta_n", "phase_eta_s"]:
            if ref.get(k) is None:
                continue
            x, y = (np.concatenate(v) if isinstance(v, list) else v for v in (got[k], ref[k]))
            assert np.array_equal(x, y, equal_nan=True), k
