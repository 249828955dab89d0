"""The sweep's input preparation on the GPU (mdz_rheo_softening, mdz_rheo_shear_modulus)
against the reference's golden fixtures and the oracle, at the fixtures' sizes and at
the 2049 x 2049 cells of the large sweep.  Piecewise-linear softening, hardening and the
shear modulus are bit for bit; the erfc softening is within the accuracy of erfc
(CUDA's on the device, the C library's in the reference: a few ulp of erfc, which the
formula carries into fric, dil and C scaled by the softening amplitude)."""
import os

import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from common import clone
from golden import cases
from test_prep_oracle import golden_prep

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
ERFC_RTOL = 1e-13  # of the field's largest magnitude


@pytest.fixture(scope="module")
def ctx():
    c = R.Context(0)
    yield c
    c.close()


def same_bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


def check_soft(got, ref, smooth, keys):
    for k in keys:
        g, r = np.asarray(got[k]), np.asarray(ref[k])
        if smooth:
            assert np.array_equal(np.isnan(g), np.isnan(r)), k
            ok = ~np.isnan(r)
            g, r = g[ok], r[ok]
            scale = max(float(np.max(np.abs(r))), 1e-300) if r.size else 1.0
            err = float(np.max(np.abs(g - r))) / scale if r.size else 0.0
            assert err <= ERFC_RTOL, (k, err)
        else:
            assert np.array_equal(np.isnan(g), np.isnan(r)), k
            ok = ~np.isnan(r)
            assert same_bits(g[ok], r[ok]), k


def to_dev(arrays):
    return {k: ([torch.from_numpy(x).cuda() for x in v] if isinstance(v, list) else torch.from_numpy(v).cuda())
            for k, v in arrays.items()}


@pytest.mark.parametrize("name", list(cases.SOFTENING_CASES))
def test_gpu_softening_matches_golden(ctx, name):
    w, g = golden_prep(name, "softening")
    _, smooth, hard, noise, _ = cases.SOFTENING_CASES[name]
    rc, st = ctx.softening(w.model, w.mat, R.PrepFieldSet(w.arrays), smooth, hard, noise)
    assert rc == R.MDZ_OK and st.kernel_launches == 1
    check_soft(w.arrays, g, smooth == 1 and hard != 1, R.SOFT_N + R.SOFT_S)


@pytest.mark.parametrize("name", list(cases.SHEAR_CASES))
def test_gpu_shear_modulus_matches_golden(ctx, name):
    w, g = golden_prep(name, "shear_modulus")
    rc, _ = ctx.shear_modulus(w.model, w.mat, R.PrepFieldSet(w.arrays))
    assert rc == R.MDZ_OK
    for k in R.MOD_N + R.MOD_S:
        assert same_bits(w.arrays[k], g[k]), k


@pytest.mark.parametrize("smooth,hard,noise,air,per", [(0, 0, 1, 0.2, 1), (1, 0, 0, 0.0, 0), (0, 1, 1, 0.3, 0)])
def test_gpu_softening_device_match_oracle_2049(ctx, smooth, hard, noise, air, per):
    w = W.prep_workload(seed=40 + smooth + 2 * hard, ncx=2049, nphases=5, air=air, periodic=per)
    ref = clone(w.arrays)
    assert O.orc_softening(w.model, w.mat, R.PrepFieldSet(ref), smooth, hard, noise) == R.MDZ_OK
    d = to_dev(w.arrays)
    rc, st = ctx.softening(w.model, w.mat, R.PrepFieldSet(d), smooth, hard, noise, mem=R.MEM_DEVICE)
    assert rc == R.MDZ_OK and st.h2d_bytes == 0
    got = {k: d[k].cpu().numpy() for k in R.SOFT_N + R.SOFT_S}
    check_soft(got, ref, smooth == 1 and hard != 1, R.SOFT_N + R.SOFT_S)


@pytest.mark.parametrize("air,per", [(0.0, 0), (0.3, 1)])
def test_gpu_shear_modulus_device_match_oracle_2049(ctx, air, per):
    w = W.prep_workload(seed=50 + per, ncx=2049, nphases=5, air=air, periodic=per)
    ref = clone(w.arrays)
    assert O.orc_shear_modulus(w.model, w.mat, R.PrepFieldSet(ref)) == R.MDZ_OK
    d = to_dev(w.arrays)
    rc, _ = ctx.shear_modulus(w.model, w.mat, R.PrepFieldSet(d), mem=R.MEM_DEVICE)
    assert rc == R.MDZ_OK
    for k in R.MOD_N + R.MOD_S:
        assert same_bits(d[k].cpu().numpy(), ref[k]), k


@pytest.mark.parametrize("smooth,hard", [(0, 0), (1, 0), (0, 1)])
def test_gpu_softening_special_strains(ctx, smooth, hard):
    """NaN, +-Inf, -0 and the exact softening bounds as plastic strain: the comparisons of
    the piecewise form run on integer keys on the GPU and must keep IEEE semantics."""
    w = W.prep_workload(seed=70, ncx=60, ncz=45, nphases=4, air=0.2)
    for key in ("strain_pl_n", "strain_pl_s"):
        st = w.arrays[key]
        st[0::9], st[1::9], st[2::9], st[3::9] = np.nan, np.inf, -np.inf, -0.0
        st[4::9], st[5::9] = w.mat.pls_start[1], w.mat.pls_end[2]
        st[6::9] = np.nextafter(w.mat.pls_end[3], -np.inf)
    ref = clone(w.arrays)
    assert O.orc_softening(w.model, w.mat, R.PrepFieldSet(ref), smooth, hard, 1) == R.MDZ_OK
    ctx.softening(w.model, w.mat, R.PrepFieldSet(w.arrays), smooth, hard, 1)
    check_soft(w.arrays, ref, smooth == 1 and hard != 1, R.SOFT_N + R.SOFT_S)


def test_gpu_shear_modulus_infinite_status(ctx):
    w = W.prep_workload(seed=15, ncx=10, ncz=8, nphases=2)
    for p in range(2):
        w.arrays["phase_perc_n"][p][17] = 0.0
        w.arrays["phase_perc_n"][p][40] = 0.0
    rc, st = ctx.shear_modulus(w.model, w.mat, R.PrepFieldSet(w.arrays), check=False)
    assert rc == R.MDZ_ESHEAR_INF and st.error_node == 17
    assert np.isinf(w.arrays["mu_n"][17])


def test_gpu_prep_async_and_errors(ctx):
    w = W.prep_workload(seed=60, ncx=70, ncz=50, nphases=3, air=0.2)
    d = to_dev(w.arrays)
    rc, _ = ctx.softening(w.model, w.mat, R.PrepFieldSet(d), mem=R.MEM_DEVICE, flags=R.SWEEP_ASYNC)
    assert rc == R.MDZ_OK
    rc, st = ctx.sync()
    assert rc == R.MDZ_OK and st.status == R.MDZ_OK
    ref = clone(w.arrays)
    O.orc_softening(w.model, w.mat, R.PrepFieldSet(ref))
    assert same_bits(d["C_s"].cpu().numpy(), ref["C_s"])
    # asynchronous calls need device memory; marker noise needs the noise fields
    rc, _ = ctx.softening(w.model, w.mat, R.PrepFieldSet(w.arrays), flags=R.SWEEP_ASYNC, check=False)
    assert rc == R.MDZ_EINVAL
    partial = dict(w.arrays)
    partial["noise_s"] = None
    rc, _ = ctx.softening(w.model, w.mat, R.PrepFieldSet(partial), marker_noise=1, check=False)
    assert rc == R.MDZ_EINVAL
