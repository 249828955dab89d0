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
from golden.make_golden import load_marker_G, load_marker_inputs, marker_opts
from test_markers_oracle import boundary_workload, tiny_weight_workload

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DIRECTOR_ULP = 4
# subgrid diffusion 2: P2Mastah's sums in another order and CUDA's exp, against the
# largest magnitude of each stress field
SUBGRID_RTOL = 1e-12


@pytest.fixture(scope="module")
def ctx():
    c = R.Context(0)
    yield c
    c.close()


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.array_equal(a.view(np.uint64), b.view(np.uint64))


def check(got_mk, got_wxz, ref_mk, ref_wxz, subgrid=False):
    for k in ("sxxd", "szzd", "sxz"):
        if subgrid:
            g, r = np.asarray(got_mk[k]), np.asarray(ref_mk[k])
            err = float(np.max(np.abs(g - r))) / float(np.max(np.abs(r)))
            assert err <= SUBGRID_RTOL, (k, err)
        else:
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
    opts = marker_opts(*cases.MARKER_CASES[name][1:], G=load_marker_G(g))
    rc, st = ctx.marker_stress(model, opts, grid, mk, dx, dz)
    assert rc == R.MDZ_OK and st.kernel_launches == (2 if opts.elastic != 1 else 5 if opts.subgrid_diffusion == 2 else 4)
    check(mk, grid["wxz"], {k: g["out_" + k] for k in ("sxxd", "szzd", "sxz", "nx", "nz")}, g["out_wxz"],
          subgrid=opts.subgrid_diffusion == 2)


@pytest.mark.parametrize("air,per,stencil,rot,sub", [(0.0, 0, 1, 1, 0), (0.3, 1, 9, 2, 0), (0.0, 0, 1, 1, 2),
                                                     (0.3, 1, 9, 2, 2)])
def test_gpu_marker_stress_device_match_oracle(ctx, air, per, stencil, rot, sub):
    w = W.marker_workload(seed=60 + stencil + sub, ncx=1025, markers_per_cell=4, air=air, periodic=per)
    opts = marker_opts(1, rot, 1, 1, stencil, sub, G=w.info["G"])
    g_ref, m_ref = copies(w)
    assert O.orc_marker_stress(w.model, opts, g_ref, m_ref, w.info["dx"], w.info["dz"]) == R.MDZ_OK
    g_h, m_h = copies(w)
    gd = {k: torch.from_numpy(v).cuda() for k, v in g_h.items()}
    md = {k: torch.from_numpy(v).cuda() for k, v in m_h.items()}
    rc, st = ctx.marker_stress(w.model, opts, gd, md, w.info["dx"], w.info["dz"], mem=R.MEM_DEVICE)
    assert rc == R.MDZ_OK and st.h2d_bytes == 0
    check({k: v.cpu().numpy() for k, v in md.items()}, gd["wxz"].cpu().numpy(), m_ref, g_ref["wxz"], subgrid=sub == 2)


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


@pytest.mark.parametrize("name", ["markers_on_boundaries", "tiny_weights"])
def test_gpu_subgrid_diffusion_edge_markers(ctx, name):
    """Subgrid diffusion on markers exactly on node coordinates and at the edge of their
    P2Mastah support."""
    w = boundary_workload() if name == "markers_on_boundaries" else tiny_weight_workload()
    opts = marker_opts(1, 1, 0, 1, 9, 2, G=w.info["G"])
    g_ref, m_ref = copies(w)
    assert O.orc_marker_stress(w.model, opts, g_ref, m_ref, w.info["dx"], w.info["dz"]) == R.MDZ_OK
    g, m = copies(w)
    ctx.marker_stress(w.model, opts, g, m, w.info["dx"], w.info["dz"])
    check(m, g["wxz"], m_ref, g_ref["wxz"], subgrid=True)


@pytest.mark.parametrize("stencil", [1, 9])
def test_gpu_subgrid_diffusion_without_relaxation_is_the_plain_update(ctx, stencil):
    """Maxwell times so long that exp(-dt/t) rounds to 1: the subgrid update must give the
    plain update bit for bit."""
    w = W.marker_workload(seed=66, ncx=300, ncz=200, markers_per_cell=4, air=0.2, periodic=1)
    w.arrays["eta_phys_s"][:] = 1e40
    g0, m0 = copies(w)
    ctx.marker_stress(w.model, marker_opts(1, 1, 1, 1, stencil), g0, m0, w.info["dx"], w.info["dz"])
    g2, m2 = copies(w)
    ctx.marker_stress(w.model, marker_opts(1, 1, 1, 1, stencil, 2, G=w.info["G"]), g2, m2, w.info["dx"],
                      w.info["dz"])
    for k in ("sxxd", "szzd", "sxz", "nx", "nz"):
        assert same(m0[k], m2[k]), k
    assert same(g0["wxz"], g2["wxz"])


def test_gpu_marker_stress_status_and_async(ctx):
    w = W.marker_workload(seed=80, ncx=30, ncz=20)
    g, m = copies(w)
    m["x"][7] = w.arrays["xg_coord"][-1] + 0.6 * w.info["dx"]
    rc, st = ctx.marker_stress(w.model, marker_opts(1, 1, 0, 1, 1), g, m, w.info["dx"], w.info["dz"], check=False)
    assert rc == R.MDZ_EMARKER_OUT and st.error_node == 7
    g, m = copies(w)
    rc, _ = ctx.marker_stress(w.model, marker_opts(1, 1, 0, 1, 1, 2), g, m, w.info["dx"], w.info["dz"], check=False)
    assert rc == R.MDZ_EINVAL  # subgrid diffusion without the shear modulus
    g, m = copies(w)
    m["x"][7] = w.info["markers"]["x"][7]
    m["phase"][11] = 5
    rc, st = ctx.marker_stress(w.model, marker_opts(1, 1, 0, 1, 1, 2, G=w.info["G"]), g, m, w.info["dx"],
                               w.info["dz"], check=False)
    assert rc == R.MDZ_EINVAL and st.error_node == 11  # a phase the model does not have
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
