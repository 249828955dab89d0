"""Edge cases of the sweep on the GPU against the oracle: one cell, one column, one row,
ragged grids, one phase, a grid of air only, periodic with two columns, a warm-started
sweep whose warps are mostly empty, a batch mixing a one-cell grid with larger ones, and
the sizes the C ABI rejects.  The oracle's own results on these grids equal the
reference's bit for bit (tests/test_oracle_vs_reference.py)."""
import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from common import RTOL, clone, worst

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = R.Context(0)
    yield c
    c.close()


def check(g, c, w, label):
    errs = worst(g, c, w.arrays, w.model)
    bad = {k: v for k, v in errs.items() if v > RTOL}
    assert not bad, f"{label}: {bad}"


EDGES = {
    "one_cell": (lambda: W.plain_large(seed=21, ncx=1, ncz=1), False),
    "one_column": (lambda: W.plain_large(seed=22, ncx=1, ncz=9), False),
    "one_row": (lambda: W.plain_large(seed=23, ncx=9, ncz=1), False),
    "ragged_3x300": (lambda: W.plain_large(seed=24, ncx=3, ncz=300), False),
    "ragged_300x3": (lambda: W.plain_large(seed=27, ncx=300, ncz=3), False),
    "one_phase": (lambda: W.plain_large(seed=25, ncx=12, ncz=10, nphases=1), False),
    "aniso_one_row": (lambda: W.aniso(seed=26, ncx=7, ncz=1), True),
}


@pytest.mark.parametrize("start", [0, R.SWEEP_REF_START])
@pytest.mark.parametrize("name", list(EDGES))
def test_edge_grids_match_oracle(ctx, name, start):
    make, aniso = EDGES[name]
    w = make()
    g, c = clone(w.arrays), clone(w.arrays)
    fn = ctx.sweep_aniso if aniso else ctx.sweep
    rc, st = fn(w.model, w.mat, R.FieldSet(g), flags=start, check=False)
    rc2, st2 = O.orc_sweep(w.model, w.mat, R.FieldSet(c), aniso=aniso)
    assert rc == rc2 == R.MDZ_OK
    assert st.phase_calls == st2.phase_calls and st.plastic_calls == st2.plastic_calls
    check(g, c, w, name)


def test_periodic_two_columns(ctx):
    w = W.plain_small(seed=28, ncx=2, ncz=5)
    w.model.periodic_x = 1
    g, c = clone(w.arrays), clone(w.arrays)
    rc, st = ctx.sweep(w.model, w.mat, R.FieldSet(g), check=False)
    rc2, _ = O.orc_sweep(w.model, w.mat, R.FieldSet(c))
    assert rc == rc2 == R.MDZ_OK
    check(g, c, w, "periodic, two columns")


def test_air_only_grid(ctx):
    """Every centroid and vertex in the air: no local solve, every output zero (the
    reference skips air nodes after zeroing them), and no error."""
    w = W.plain_large(seed=29, ncx=12, ncz=10)
    w.arrays["BCp_type"][:] = 30
    w.arrays["BCg_type"][:] = 30
    g, c = clone(w.arrays), clone(w.arrays)
    rc, st = ctx.sweep(w.model, w.mat, R.FieldSet(g), check=False)
    rc2, st2 = O.orc_sweep(w.model, w.mat, R.FieldSet(c))
    assert rc == rc2 == R.MDZ_OK and st.phase_calls == st2.phase_calls == 0
    for k in R.CEN_OUT + R.VER_OUT:
        if g.get(k) is not None and not isinstance(g[k], list):
            assert np.array_equal(g[k], c[k], equal_nan=True), k


def test_sizes_the_abi_rejects(ctx):
    w = W.plain_large(seed=30, ncx=4, ncz=4)
    for nx, nz in ((1, 5), (5, 1), (0, 0)):
        m = w.model
        keep = (m.Nx, m.Nz)
        m.Nx, m.Nz = nx, nz
        rc, _ = ctx.sweep(m, w.mat, R.FieldSet(clone(w.arrays)), check=False)
        m.Nx, m.Nz = keep
        assert rc == R.MDZ_EINVAL, (nx, nz, rc)


@pytest.fixture(scope="module")
def network(ctx):
    import mdz_warmstart as WS
    X, Y = WS.collect(ctx, [W.plain_large(seed=160, ncx=97)])
    w, _, _ = WS.train(ctx, X, Y, WS.FEAT_ISO, WS.default_cfg(epochs=2, batch=4096))
    return w


@pytest.mark.parametrize("name", ["one_cell", "one_row", "ragged_3x300"])
def test_warm_start_on_mostly_empty_warps(ctx, network, name):
    """Warps with 1 to 9 valid lanes still evaluate the network together (the lanes past
    the end feed zeros); the warm-started results meet the oracle's."""
    ctx.set_warmstart(network, R.DEFAULT_START)
    w = EDGES[name][0]()
    g, c = clone(w.arrays), clone(w.arrays)
    rc, st = ctx.sweep(w.model, w.mat, R.FieldSet(g), flags=R.SWEEP_WARMSTART, check=False)
    rc2, st2 = O.orc_sweep(w.model, w.mat, R.FieldSet(c))
    assert rc == rc2 == R.MDZ_OK and st.mma_fault == 0 and st.phase_calls == st2.phase_calls
    check(g, c, w, f"warm {name}")
    ctx.set_warmstart(None, R.DEFAULT_START)


def test_batch_with_a_one_cell_grid(ctx):
    torch = pytest.importorskip("torch")
    ws = [W.plain_large(seed=31, ncx=1, ncz=1), W.plain_small(seed=32, ncx=33, ncz=7),
          W.plain_large(seed=33, ncx=1, ncz=40)]
    devs = [{k: ([torch.from_numpy(x.copy()).cuda() for x in v] if isinstance(v, list)
                 else torch.from_numpy(v.copy()).cuda()) for k, v in w.arrays.items()} for w in ws]
    b = R.Batch(ctx, [w.model for w in ws], [w.mat for w in ws], [R.FieldSet(d) for d in devs])
    rc, st = b.sweep()
    assert rc == R.MDZ_OK
    b.close()
    for w, d in zip(ws, devs):
        g = {k: ([x.cpu().numpy() for x in v] if isinstance(v, list) else v.cpu().numpy()) for k, v in d.items()}
        c = clone(w.arrays)
        assert O.orc_sweep(w.model, w.mat, R.FieldSet(c))[0] == R.MDZ_OK
        check(g, c, w, f"batch grid {w.model.Nx - 1}x{w.model.Nz - 1}")
