"""StrainRateComponents on the GPU (mdz_rheo_strain_rates) against the reference's
golden fixtures and the oracle: bit for bit, at the fixtures' sizes and at the
2049 x 2049 cells of the large sweep, in host and device memory, and chained with
the sweep on device-resident fields as UpdateNonLinearity does."""
import os

import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from common import clone
from golden import cases

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ctx():
    c = R.Context(0)
    yield c
    c.close()


def same_bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


def to_dev(arrays):
    return {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in arrays.items()}


@pytest.mark.parametrize("name", list(cases.STRAIN_CASES))
def test_gpu_strain_rates_match_golden(ctx, name):
    builder, oop, comp = cases.STRAIN_CASES[name]
    w = builder()
    g = np.load(os.path.join(GOLDEN, f"strain_rates_{name}.npz"))
    rc, st = ctx.strain_rates(w.model, w.info["dx"], w.info["dz"], w.arrays, out_of_plane=oop, compressible=comp)
    assert rc == R.MDZ_OK and st.kernel_launches == 1
    for k in R.SR_N + R.SR_S:
        assert same_bits(w.arrays[k], g[k]), k


@pytest.mark.parametrize("ncx,ncz,air,per,oop,comp", [
    (2049, 2049, 0.0, 0, 0, 0.0),   # the large sweep's grid
    (517, 301, 0.3, 1, 1, 1.0),     # air, periodic, out of plane, compressible
    (33, 1000, 0.2, 0, 0, 0.5),     # tall and narrow: partial tiles in x
])
def test_gpu_strain_rates_device_match_oracle(ctx, ncx, ncz, air, per, oop, comp):
    w = W.velocity_field(seed=ncx + ncz, ncx=ncx, ncz=ncz, air=air, periodic=per)
    ref = {k: v.copy() for k, v in w.arrays.items()}
    assert O.orc_strain_rates(w.model, w.info["dx"], w.info["dz"], ref, oop, comp) == R.MDZ_OK
    d = to_dev(w.arrays)
    rc, st = ctx.strain_rates(w.model, w.info["dx"], w.info["dz"], d, out_of_plane=oop, compressible=comp,
                              mem=R.MEM_DEVICE)
    assert rc == R.MDZ_OK
    assert st.h2d_bytes == 0 and st.d2h_bytes == 0
    for k in R.SR_N + R.SR_S:
        assert same_bits(d[k].cpu().numpy(), ref[k]), k


@pytest.mark.parametrize("v0,L", [(1e303, 1e3), (1e-300, 1e7), (3e-308, 1e3)])
def test_gpu_strain_rates_extreme_magnitudes(ctx, v0, L):
    """Rates near overflow and in the subnormal range take the kernel's exact
    reference-order averaging; the results stay bitwise those of the oracle."""
    w = W.velocity_field(seed=41, ncx=90, ncz=70, air=0.2, v0=v0, L=L)
    ref = {k: v.copy() for k, v in w.arrays.items()}
    assert O.orc_strain_rates(w.model, w.info["dx"], w.info["dz"], ref, 1, 1.0) == R.MDZ_OK
    ctx.strain_rates(w.model, w.info["dx"], w.info["dz"], w.arrays, out_of_plane=1, compressible=1.0)
    for k in R.SR_N + R.SR_S:
        assert same_bits(w.arrays[k], ref[k]), k


def test_gpu_strain_rates_async_and_errors(ctx):
    w = W.velocity_field(seed=3, ncx=70, ncz=50, air=0.2)
    d = to_dev(w.arrays)
    rc, _ = ctx.strain_rates(w.model, w.info["dx"], w.info["dz"], d, mem=R.MEM_DEVICE, flags=R.SWEEP_ASYNC)
    assert rc == R.MDZ_OK
    rc, st = ctx.sync()
    assert rc == R.MDZ_OK and st.status == R.MDZ_OK
    ref = {k: v.copy() for k, v in w.arrays.items()}
    O.orc_strain_rates(w.model, w.info["dx"], w.info["dz"], ref, 0, 0.0)
    assert same_bits(d["exxd_s"].cpu().numpy(), ref["exxd_s"])
    # asynchronous calls need device memory; every array must be given
    rc, _ = ctx.strain_rates(w.model, w.info["dx"], w.info["dz"], w.arrays, flags=R.SWEEP_ASYNC, check=False)
    assert rc == R.MDZ_EINVAL
    partial = dict(w.arrays)
    partial["wxz_n"] = None
    rc, _ = ctx.strain_rates(w.model, w.info["dx"], w.info["dz"], partial, check=False)
    assert rc == R.MDZ_EINVAL


def test_gpu_update_nonlinearity_on_device(ctx):
    """Strain rates written straight into the sweep's device-resident inputs, then the
    sweep (UpdateNonLinearity, StokesRoutines.c:55-62), against the same sweep fed with
    the oracle's strain rates from host memory: the strain rates are bitwise equal, so
    the two sweeps must agree bitwise."""
    ncx, ncz = 96, 80
    g = W.plain_large(seed=31, ncx=ncx, ncz=ncz)
    v = W.velocity_field(seed=32, ncx=ncx, ncz=ncz, v0=3e-10)
    dx, dz = v.info["dx"], v.info["dz"]
    # host path: oracle strain rates -> host sweep
    hv = {k: a.copy() for k, a in v.arrays.items()}
    hv["BCp_type"], hv["BCg_type"] = g.arrays["BCp_type"], g.arrays["BCg_type"]
    assert O.orc_strain_rates(g.model, dx, dz, hv, 0, 0.0) == R.MDZ_OK
    host = clone(g.arrays)
    for k in R.SR_N + R.SR_S:
        if k in host:
            host[k][:] = hv[k]
    ctx.sweep(g.model, g.mat, R.FieldSet(host))
    # device path: strain rates into the sweep's own device buffers, then the sweep
    d = {k: ([torch.from_numpy(x).cuda() for x in a] if isinstance(a, list) else torch.from_numpy(a).cuda())
         for k, a in clone(g.arrays).items()}
    sr = {k: d[k] for k in R.SR_N + R.SR_S if k in d}
    sr.update({"u_in": torch.from_numpy(v.arrays["u_in"]).cuda(), "v_in": torch.from_numpy(v.arrays["v_in"]).cuda(),
               "BCp_type": d["BCp_type"], "BCg_type": d["BCg_type"],
               "wxz": torch.zeros(g.Nv, dtype=torch.float64, device="cuda"),
               "wxz_n": torch.zeros(g.Nc, dtype=torch.float64, device="cuda")})
    ctx.strain_rates(g.model, dx, dz, sr, mem=R.MEM_DEVICE)
    ctx.sweep(g.model, g.mat, R.FieldSet(d), mem=R.MEM_DEVICE)
    for k in ("eta_n", "eta_s", "sxxd", "szzd", "sxz", "sxxd_s", "eII_pl"):
        assert same_bits(d[k].cpu().numpy(), host[k]), k
