"""P2Mastah for marker arrays on the GPU (mdz_rheo_p2mastah) against the restatement:
the nodes written and the nodes kept are the same, and the written values agree within
1e-13 of the field's scale -- the sums run in another order (FP64 atomics), as the
reference's own sums do when its thread count changes."""
import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from test_p2mastah_oracle import CASES, p2m_case

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
RTOL = 1e-13


@pytest.fixture(scope="module")
def ctx():
    c = R.Context(0)
    yield c
    c.close()


def close(got, ref, kept):
    """`kept`: the initial values; nodes the reference left alone must be unchanged bit for bit."""
    untouched = ref.view(np.uint64) == kept.view(np.uint64)
    assert np.array_equal(got[untouched].view(np.uint64), ref[untouched].view(np.uint64))
    w = ~untouched
    if w.any():
        err = float(np.max(np.abs(got[w] - ref[w]))) / float(np.max(np.abs(ref[w])))
        assert err <= RTOL, err


@pytest.mark.parametrize("stencil", [1, 9])
@pytest.mark.parametrize("avg", [0, 1, 2])
@pytest.mark.parametrize("case", list(CASES))
def test_gpu_p2mastah_matches_oracle(ctx, case, avg, stencil):
    seed, ncx, ncz, mpc, air, per = CASES[case]
    w, values, nn, ns = p2m_case(seed, ncx, ncz, mpc, air, per, on_nodes=(case == "on_nodes"))
    rn, rs = nn.copy(), ns.copy()
    assert O.orc_p2mastah(w.model, w.arrays, w.info["markers"], values, avg, stencil, rn, rs, w.info["dx"],
                          w.info["dz"]) == R.MDZ_OK
    gn, gs = nn.copy(), ns.copy()
    rc, st = ctx.p2mastah(w.model, w.arrays, w.info["markers"], values, avg, stencil, gn, gs, w.info["dx"],
                          w.info["dz"])
    assert rc == R.MDZ_OK and st.kernel_launches == 2
    close(gn, rn, nn)
    close(gs, rs, ns)


@pytest.mark.parametrize("stencil", [1, 9])
def test_gpu_p2mastah_large_device(ctx, stencil):
    """1025 x 1025 cells, 16 markers per cell, device memory, one grid at a time."""
    w = W.marker_workload(seed=37, ncx=1025, markers_per_cell=16, air=0.2, periodic=1)
    rng = np.random.default_rng(38)
    values = rng.uniform(0.0, 1.5, w.info["markers"]["x"].size)
    nn = np.zeros((w.model.Nx - 1) * (w.model.Nz - 1))
    ns = np.zeros(w.model.Nx * w.model.Nz)
    rn, rs = nn.copy(), ns.copy()
    O.orc_p2mastah(w.model, w.arrays, w.info["markers"], values, 0, stencil, rn, rs, w.info["dx"], w.info["dz"])
    gd = {k: torch.from_numpy(v).cuda() for k, v in w.arrays.items()}
    md = {k: torch.from_numpy(v).cuda() for k, v in w.info["markers"].items()}
    vd, gn = torch.from_numpy(values).cuda(), torch.from_numpy(nn.copy()).cuda()
    rc, st = ctx.p2mastah(w.model, gd, md, vd, 0, stencil, gn, None, w.info["dx"], w.info["dz"], mem=R.MEM_DEVICE)
    assert rc == R.MDZ_OK and st.h2d_bytes == 0
    gs = torch.from_numpy(ns.copy()).cuda()
    ctx.p2mastah(w.model, gd, md, vd, 0, stencil, None, gs, w.info["dx"], w.info["dz"], mem=R.MEM_DEVICE)
    close(gn.cpu().numpy(), rn, nn)
    close(gs.cpu().numpy(), rs, ns)


def test_gpu_p2mastah_status(ctx):
    w, values, nn, ns = p2m_case(39, 12, 10, 2, 0.0, 0)
    w.info["markers"]["phase"][5] = 9
    rc, st = ctx.p2mastah(w.model, w.arrays, w.info["markers"], values, 0, 1, nn, ns, w.info["dx"], w.info["dz"],
                          check=False)
    assert rc == R.MDZ_EINVAL and st.error_node == 5
    rc, _ = ctx.p2mastah(w.model, w.arrays, w.info["markers"], values, 3, 1, nn, ns, w.info["dx"], w.info["dz"],
                         check=False)
    assert rc == R.MDZ_EINVAL
