"""UpdateParticleStress on the GPU (mdz_rheo_marker_stress) against the reference's
golden fixtures and the oracle.  Marker stresses and the rewritten wxz are bit for bit;
the director agrees to a few ulp (its normalisation squares by multiplication where the
reference calls pow)."""
import os

import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from golden import cases
from golden.make_golden import load_marker_inputs, marker_opts
from test_markers_oracle import boundary_workload, tiny_weight_workload

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DIRECTOR_ULP = 4


@pytest.fixture(scope="module")
def ctx():
    c = R.Context(0)
    yield c
    c.close()


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.array_equal(a.view(np.uint64), b.view(np.uint64))


def check(got_mk, got_wxz, ref_mk, ref_wxz):
    for k in ("sxxd", "szzd", "sxz"):
        assert same(got_mk[k], ref_mk[k]), k
    assert same(got_wxz, ref_wxz)
    for k in ("nx", "nz"):
        g, r = np.asarray(got_mk[k]), np.asarray(ref_mk[k])
        ulps = np.abs(g - r) / np.spacing(np.maximum(np.abs(r), 1e-300))
        assert float(ulps.max()) <= DIRECTOR_ULP, (k, float(ulps.max()))


def copies(w):
    return {k: v.copy() for k, v in w.arrays.items()}, {k: v.copy() for k, v in w.info["markers"].items()}


@pytest.mark.parametrize("name", list(cases.MARKER_CASES))
def test_gpu_marker_stress_matches_golden(ctx, name):
    g = np.load(os.path.join(GOLDEN, f"markers_{name}.npz"))
    model, grid, mk, dx, dz = load_marker_inputs(g)
    opts = marker_opts(*cases.MARKER_CASES[name][1:])
    rc, st = ctx.marker_stress(model, opts, grid, mk, dx, dz)
    assert rc == R.MDZ_OK and st.kernel_launches == (4 if opts.elastic == 1 else 2)
    check(mk, grid["wxz"], {k: g["out_" + k] for k in ("sxxd", "szzd", "sxz", "nx", "nz")}, g["out_wxz"])


@pytest.mark.parametrize("air,per,stencil,rot", [(0.0, 0, 1, 1), (0.3, 1, 9, 2)])
def test_gpu_marker_stress_device_match_oracle(ctx, air, per, stencil, rot):
    w = W.marker_workload(seed=60 + stencil, ncx=1025, markers_per_cell=4, air=air, periodic=per)
    opts = marker_opts(1, rot, 1, 1, stencil)
    g_ref, m_ref = copies(w)
    assert O.orc_marker_stress(w.model, opts, g_ref, m_ref, w.info["dx"], w.info["dz"]) == R.MDZ_OK
    g_h, m_h = copies(w)
    gd = {k: torch.from_numpy(v).cuda() for k, v in g_h.items()}
    md = {k: torch.from_numpy(v).cuda() for k, v in m_h.items()}
    rc, st = ctx.marker_stress(w.model, opts, gd, md, w.info["dx"], w.info["dz"], mem=R.MEM_DEVICE)
    assert rc == R.MDZ_OK and st.h2d_bytes == 0
    check({k: v.cpu().numpy() for k, v in md.items()}, gd["wxz"].cpu().numpy(), m_ref, g_ref["wxz"])


def test_gpu_markers_on_cell_boundaries(ctx):
    w = boundary_workload()
    opts = marker_opts(1, 1, 1, 1, 9)
    g_ref, m_ref = copies(w)
    assert O.orc_marker_stress(w.model, opts, g_ref, m_ref, w.info["dx"], w.info["dz"]) == R.MDZ_OK
    g, m = copies(w)
    ctx.marker_stress(w.model, opts, g, m, w.info["dx"], w.info["dz"])
    check(m, g["wxz"], m_ref, g_ref["wxz"])


@pytest.mark.parametrize("stencil", [1, 9])
def test_gpu_tiny_weights_take_the_exact_sums(ctx, stencil):
    """P2Mastah weights below 1e-30 that are not zero: the exact per-vertex sums, as the
    reference forms them, decide which vertices keep wxz."""
    w = tiny_weight_workload()
    opts = marker_opts(1, 1, 0, 1, stencil)
    g_ref, m_ref = copies(w)
    assert O.orc_marker_stress(w.model, opts, g_ref, m_ref, w.info["dx"], w.info["dz"]) == R.MDZ_OK
    g, m = copies(w)
    ctx.marker_stress(w.model, opts, g, m, w.info["dx"], w.info["dz"])
    check(m, g["wxz"], m_ref, g_ref["wxz"])
    assert np.sum(g_ref["wxz"] == w.arrays["wxz"]) > 0


def test_gpu_marker_stress_status_and_async(ctx):
    w = W.marker_workload(seed=80, ncx=30, ncz=20)
    g, m = copies(w)
    m["x"][7] = w.arrays["xg_coord"][-1] + 0.6 * w.info["dx"]
    rc, st = ctx.marker_stress(w.model, marker_opts(1, 1, 0, 1, 1), g, m, w.info["dx"], w.info["dz"], check=False)
    assert rc == R.MDZ_EMARKER_OUT and st.error_node == 7
    o = marker_opts(1, 1, 0, 1, 1)
    o.subgrid_diffusion = 2
    g, m = copies(w)
    rc, _ = ctx.marker_stress(w.model, o, g, m, w.info["dx"], w.info["dz"], check=False)
    assert rc == R.MDZ_EUNSUPPORTED
    g, m = copies(w)
    gd = {k: torch.from_numpy(v).cuda() for k, v in g.items()}
    md = {k: torch.from_numpy(v).cuda() for k, v in m.items()}
    rc, _ = ctx.marker_stress(w.model, marker_opts(1, 2, 1, 1, 1), gd, md, w.info["dx"], w.info["dz"],
                              mem=R.MEM_DEVICE, flags=R.SWEEP_ASYNC)
    assert rc == R.MDZ_OK
    rc, st = ctx.sync()
    assert rc == R.MDZ_OK and st.status == R.MDZ_OK
    g_ref, m_ref = copies(w)
    O.orc_marker_stress(w.model, marker_opts(1, 2, 1, 1, 1), g_ref, m_ref, w.info["dx"], w.info["dz"])
    check({k: v.cpu().numpy() for k, v in md.items()}, gd["wxz"].cpu().numpy(), m_ref, g_ref["wxz"])
