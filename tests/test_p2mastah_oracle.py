"""P2Mastah for marker arrays (ParticleRoutines.c:2170-2665) on the CPU: the C
restatement against the reference's own function, run on one OpenMP thread so that its
per-thread partial sums run in marker order -- bit for bit on the centroids and the
vertices, for the three averages, both stencils, periodic x and air."""
import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from test_markers_oracle import boundary_workload

need_ref = pytest.mark.skipif(O.reference() is None, reason="reference build absent (oracle/_ref)")


def p2m_case(seed, ncx, ncz, mpc, air, periodic, on_nodes=False):
    w = boundary_workload() if on_nodes else W.marker_workload(seed=seed, ncx=ncx, ncz=ncz, markers_per_cell=mpc,
                                                                air=air, periodic=periodic)
    rng = np.random.default_rng(seed + 100)
    values = rng.uniform(0.05, 2.0, w.info["markers"]["x"].size)
    nn = rng.standard_normal((w.model.Nx - 1) * (w.model.Nz - 1))
    ns = rng.standard_normal(w.model.Nx * w.model.Nz)
    return w, values, nn, ns


CASES = {
    "plain": (31, 23, 19, 4, 0.0, 0),
    "air_periodic": (32, 20, 17, 6, 0.25, 1),
    "one_marker_per_cell": (33, 15, 21, 1, 0.1, 0),
    "on_nodes": (34, 0, 0, 0, 0.0, 0),
}


def run(fn, case, avg, stencil):
    seed, ncx, ncz, mpc, air, per = CASES[case]
    w, values, nn, ns = p2m_case(seed, ncx, ncz, mpc, air, per, on_nodes=(case == "on_nodes"))
    n, s = nn.copy(), ns.copy()
    rc = fn(w.model, w.arrays, w.info["markers"], values, avg, stencil, n, s, w.info["dx"], w.info["dz"])
    return rc, n, s, nn, ns


@need_ref
@pytest.mark.parametrize("stencil", [1, 9])
@pytest.mark.parametrize("avg", [0, 1, 2])
@pytest.mark.parametrize("case", list(CASES))
def test_p2mastah_restatement_is_the_reference(case, avg, stencil):
    ra, na, sa, n0, s0 = run(O.ref_p2mastah, case, avg, stencil)
    rb, nb, sb, _, _ = run(O.orc_p2mastah, case, avg, stencil)
    assert ra == 0 and rb == R.MDZ_OK
    assert np.array_equal(na.view(np.uint64), nb.view(np.uint64))
    assert np.array_equal(sa.view(np.uint64), sb.view(np.uint64))
    assert np.any(na != n0) and np.any(sa != s0)


def test_p2mastah_constant_field_and_kept_nodes():
    """A constant marker value comes back as that constant wherever P2Mastah writes (all
    three averages); air nodes keep their previous values."""
    w, values, nn, ns = p2m_case(35, 18, 16, 4, 0.3, 1)
    values[:] = 0.7
    for avg in (0, 1, 2):
        n, s = nn.copy(), ns.copy()
        assert O.orc_p2mastah(w.model, w.arrays, w.info["markers"], values, avg, 9, n, s, w.info["dx"],
                              w.info["dz"]) == R.MDZ_OK
        airn = np.isin(w.arrays["BCp_type"], (30, 31))
        airs = np.isin(w.arrays["BCg_type"], (30, 31))
        assert np.array_equal(n[airn], nn[airn])
        assert np.allclose(n[~airn], 0.7, rtol=1e-15, atol=0)
        # vertex rows: periodic ends average with a neighbouring air row's kept value only where air
        inner = ~airs
        inner.reshape(w.model.Nz, w.model.Nx)[:, [0, -1]] = False
        assert np.allclose(s[inner], 0.7, rtol=1e-15, atol=0)


def test_p2mastah_rejects_unknown_phases():
    w, values, nn, ns = p2m_case(36, 10, 10, 2, 0.0, 0)
    w.info["markers"]["phase"][4] = 7
    assert O.orc_p2mastah(w.model, w.arrays, w.info["markers"], values, 0, 1, nn, ns, w.info["dx"],
                          w.info["dz"]) == R.MDZ_EINVAL
