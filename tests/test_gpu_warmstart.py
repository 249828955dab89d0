"""Learned warm start on the GPU: tensor-core network against its float64 statement,
training, the collecting sweep, and parity of warm-started sweeps with the oracle.

The warm start only moves the point where the FP64 Newton iteration starts; the
iteration still runs to the reference's residual tolerance (|r| < 1e-13 Eii,
MDLIB/RheologyDensity.c:154,172), so warm-started sweeps are held to the same parity
bar against the oracle as the plain kernel.
"""
import numpy as np
import pytest

import mdz_rheo as R
import mdz_warmstart as WS
import mdz_workloads as W
import mlp_oracle as MO
import oracle_lib as O
from common import RTOL, clone, node_Eii, worst

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = R.Context(0)
    yield c
    c.close()


def random_weights(rng, n_feat=10, X=None):
    w = R.MlpWeights()
    w.n_feat = n_feat
    a = w.arrays()
    a["W1"][:, :n_feat] = rng.uniform(-1, 1, (64, n_feat)) * np.sqrt(6.0 / n_feat)
    a["W2"][:] = rng.uniform(-1, 1, (64, 64)) * np.sqrt(6.0 / 64)
    a["W3"][:] = rng.uniform(-1, 1, (2, 64)) * 0.3
    a["b1"][:] = rng.uniform(-0.1, 0.1, 64)
    a["b2"][:] = rng.uniform(-0.1, 0.1, 64)
    a["b3"][:] = rng.uniform(-0.1, 0.1, 2)
    if X is not None:
        a["x_shift"][:n_feat] = X[:, :n_feat].mean(0)
        a["x_scale"][:n_feat] = 1.0 / X[:, :n_feat].std(0)
    else:
        a["x_scale"][:n_feat] = 1.0
    w.z_shift, w.z_scale = 1.5, 2.0
    return w


def synthetic(rng, n, n_feat=10):
    X = np.zeros((n, R.MLP_IN), np.float32)
    X[:, :n_feat] = rng.normal(size=(n, n_feat)) * rng.uniform(0.5, 3.0, n_feat) + rng.normal(size=n_feat)
    Y = np.zeros((n, 2), np.float32)
    Y[:, 0] = np.sin(X[:, 0]) + 0.3 * X[:, 1] ** 2 - 0.5 * X[:, 2] * X[:, 3] + 3.0
    Y[:, 1] = (X[:, 4] + X[:, 5] > 0.5).astype(np.float32)
    return X, Y


def rel_norm(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("n", [128, 1000, 20000])
def test_mlp_gradient_matches_float64_statement(ctx, n):
    rng = np.random.default_rng(n)
    X, Y = synthetic(rng, n)
    w = random_weights(rng, 10, X)
    g, loss = ctx.mlp_gradient(w, X, Y, w_pl=0.5)
    Wd = MO.weights(w)
    ref_q, lref_q = MO.gradient(Wd, X, Y, 0.5, bf=True)
    ref_x, lref_x = MO.gradient(Wd, X, Y, 0.5, bf=False)
    ga = g.arrays()
    for k in ["W1", "b1", "W2", "b2", "W3", "b3"]:
        gk = ga[k][:, :10] if k == "W1" else ga[k]
        rq = ref_q[k][:, :10] if k == "W1" else ref_q[k]
        rx = ref_x[k][:, :10] if k == "W1" else ref_x[k]
        eq, ex = rel_norm(gk, rq), rel_norm(gk, rx)
        print(f"n={n} {k}: vs bf16-rounded statement {eq:.2e}, vs exact float64 {ex:.2e}")
        assert eq < 5e-3, k      # FP32 accumulation order only
        assert ex < 5e-2, k      # BF16 operands
    assert np.all(ga["W1"][:, 10:] == 0.0)
    assert np.allclose(loss, lref_q, rtol=1e-3)
    assert np.allclose(loss, lref_x, rtol=3e-2)


def test_mlp_predict_matches_float64_statement(ctx):
    rng = np.random.default_rng(3)
    X, _ = synthetic(rng, 777, 12)
    w = random_weights(rng, 12, X)
    Yp = ctx.mlp_predict(w, X)
    Wd = MO.weights(w)
    ref = MO.predict(Wd, X, bf=True)
    ref_x = MO.predict(Wd, X, bf=False)
    err = np.abs(Yp - ref) / (1.0 + np.abs(ref))
    print("predict: max err vs bf16 statement", err.max(), "median", np.median(err),
          "vs float64", (np.abs(Yp - ref_x) / (1 + np.abs(ref_x))).max())
    # the hidden activations are FP32 sums rounded to BF16; where a sum lies within FP32
    # accumulation noise of a rounding tie the two sides differ by one BF16 ulp (2^-8)
    assert np.median(err) < 1e-6
    assert err.max() < 3e-3
    assert (np.abs(Yp - ref_x) / (1.0 + np.abs(ref_x))).max() < 5e-2


def test_training_fits_a_smooth_target(ctx):
    rng = np.random.default_rng(11)
    X, Y = synthetic(rng, 220_000)
    X, Y, Xt, Yt = X[:200_000], Y[:200_000], X[200_000:], Y[200_000:]
    cfg = WS.default_cfg(epochs=8, batch=4096, lr=3e-3, seed=5)
    w, loss = ctx.train_mlp(X, Y, 10, cfg)
    print("loss per epoch", loss)
    assert np.all(np.isfinite(loss))
    assert loss[-1] < 0.25 * loss[0]
    Yp = ctx.mlp_predict(w, Xt)
    z_rmse = np.sqrt(np.mean((Yp[:, 0] - Yt[:, 0]) ** 2)) / np.std(Yt[:, 0])
    acc = np.mean((Yp[:, 1] > 0.5) == (Yt[:, 1] > 0.5))
    print("held-out normalised rmse", z_rmse, "plastic accuracy", acc)
    assert z_rmse < 0.3 and acc > 0.9
    # the same seed gives the same initialisation and sample order, and each step adds its
    # CTAs' gradient sums in CTA order: a second run gives the same weights bit for bit (the
    # reported loss is an FP32 atomic sum, so it agrees closely)
    w2, loss2 = ctx.train_mlp(X, Y, 10, cfg)
    assert np.allclose(loss, loss2, rtol=2e-2)
    for k in ("W1", "W2", "W3", "b1", "b2", "b3"):
        assert np.array_equal(np.ctypeslib.as_array(getattr(w, k)), np.ctypeslib.as_array(getattr(w2, k))), k


def test_collecting_sweep_is_the_plain_sweep(ctx):
    w = W.plain_large(seed=21, ncx=64, ncz=48)
    a, b = clone(w.arrays), clone(w.arrays)
    ctx.sweep(w.model, w.mat, R.FieldSet(a), flags=R.SWEEP_REF_START)
    items = w.mat.Nb_phases * w.nodes
    X = np.empty((items, R.MLP_IN), np.float32)
    Y = np.empty((items, 2), np.float32)
    st = ctx.collect(w.model, w.mat, R.FieldSet(b), X, Y)
    for k in R.CEN_OUT + R.VER_OUT:
        if a.get(k) is not None:
            assert np.array_equal(a[k], b[k], equal_nan=True), k
    fin = np.isfinite(Y[:, 0])
    assert fin.sum() == st.phase_calls
    assert np.all(Y[fin, 0] > -1e-6)           # the converged viscosity lies below the start
    assert set(np.unique(Y[fin, 1])) <= {0.0, 1.0}
    # feature 0 is ln Eii (physical units) of the node
    Eii = np.concatenate([node_Eii(w.arrays, w.model, "n"), node_Eii(w.arrays, w.model, "s")])
    lnE = np.tile(np.log(Eii * w.model.scale_E), w.mat.Nb_phases)
    assert np.allclose(X[fin, 0], lnE[fin], atol=1e-4)


@pytest.fixture(scope="module")
def trained_iso(ctx):
    X, Y = WS.collect(ctx, [W.plain_large(seed=s, ncx=257) for s in (120, 121)])
    w, loss, _ = WS.train(ctx, X, Y, WS.FEAT_ISO, WS.default_cfg(epochs=6, batch=4096))
    return w


def run_pair(ctx, w, flags, aniso=False):
    g, c = clone(w.arrays), clone(w.arrays)
    fn = ctx.sweep_aniso if aniso else ctx.sweep
    rc, st = fn(w.model, w.mat, R.FieldSet(g), flags=flags, check=False)
    rc2, st2 = O.orc_sweep(w.model, w.mat, R.FieldSet(c), aniso=aniso)
    return rc, st, g, rc2, st2, c


def check_close(g, c, label, w):
    errs = worst(g, c, w.arrays, w.model)
    bad = {k: v for k, v in errs.items() if v > RTOL}
    print(label, "max scaled error", max(errs.values()))
    assert not bad, f"{label}: fields above {RTOL}: {bad}"


WARM_FORMS = {"per_warp": R.SWEEP_WARMSTART, "tcgen05_tiles": R.SWEEP_WARMSTART | R.SWEEP_WARM_TILES,
              "no_network": 0}


@pytest.mark.parametrize("form", list(WARM_FORMS))
def test_warm_sweep_matches_oracle(ctx, trained_iso, form):
    ctx.set_warmstart(trained_iso, R.DEFAULT_START)
    w = W.plain_large(seed=1, ncx=129)
    rc, st, g, rc2, st2, c = run_pair(ctx, w, WARM_FORMS[form])
    assert rc == rc2 == R.MDZ_OK and st.mma_fault == 0
    assert st.phase_calls == st2.phase_calls
    check_close(g, c, f"warm {form}", w)


def test_warm_start_saves_newton_iterations(ctx, trained_iso):
    """The learned start against the reference's: at most half the FP64 Newton evaluations
    (the network's guess, FP32 Newton steps, then the double-float Halley step), and what
    the network itself adds: fewer FP32 steps than the same start without it."""
    ctx.set_warmstart(trained_iso, R.DEFAULT_START)
    w = W.plain_large(seed=1, ncx=257)
    plain = WS.iterations(ctx, w, R.SWEEP_REF_START)
    default = WS.iterations(ctx, w, 0)
    warm = WS.iterations(ctx, w, R.SWEEP_WARMSTART)
    tiles = WS.iterations(ctx, w, R.SWEEP_WARMSTART | R.SWEEP_WARM_TILES)
    print("mean FP64 Newton evaluations: reference start", plain, "default start", default,
          "network (per warp)", warm, "network (tcgen05 tiles)", tiles)
    assert warm["phase_calls"] == plain["phase_calls"]
    assert warm["mean_iters"] <= 0.5 * plain["mean_iters"]
    assert tiles["mean_iters"] <= 0.5 * plain["mean_iters"]
    # the network's own gain over the same start without it: no more FP64 evaluations
    # (from its guess the few solves that the start without it leaves unresolved converge at
    # the first one), no more FP32 steps
    assert warm["mean_iters"] <= default["mean_iters"]
    assert warm["max_iters"] <= default["max_iters"]
    assert warm["mean_fp32_steps"] <= default["mean_fp32_steps"]
    assert warm["mma_fault"] == 0 and tiles["mma_fault"] == 0


def test_aniso_warm_sweep_matches_oracle(ctx):
    X, Y = WS.collect(ctx, [W.aniso(seed=130, ncx=257)], aniso=True)
    wts, _, _ = WS.train(ctx, X, Y, WS.FEAT_ANISO, WS.default_cfg(epochs=4, batch=4096))
    ctx.set_warmstart(wts, R.DEFAULT_START)
    w = W.aniso(seed=4, ncx=96)
    for form in ("per_warp", "tcgen05_tiles"):
        rc, st, g, rc2, st2, c = run_pair(ctx, w, WARM_FORMS[form], aniso=True)
        assert rc == rc2 == R.MDZ_OK and st.mma_fault == 0
        check_close(g, c, f"aniso warm {form}", w)
    plain = WS.iterations(ctx, w, R.SWEEP_REF_START, aniso=True)
    default = WS.iterations(ctx, w, 0, aniso=True)
    warm = WS.iterations(ctx, w, R.SWEEP_WARMSTART, aniso=True)
    print("aniso mean Newton iterations: reference start", plain, "default start", default, "network", warm)
    assert warm["mean_iters"] <= 0.5 * plain["mean_iters"]
    assert warm["mean_iters"] <= default["mean_iters"]


@pytest.mark.parametrize("aniso", [False, True])
def test_tcgen05_wait_that_gives_up_keeps_the_start_without_network(ctx, trained_iso, aniso):
    """The tcgen05 form's completion waits are bounded.  With a limit of 0 polls every wait
    gives up at once: the kernel records the fault, takes no tensor-memory reads while an
    MMA may be in flight, keeps the start without the network, waits for its last MMA
    before freeing tensor memory, and returns; the context stays usable."""
    if aniso:
        X, Y = WS.collect(ctx, [W.aniso(seed=131, ncx=97)], aniso=True)
        wts, _, _ = WS.train(ctx, X, Y, WS.FEAT_ANISO, WS.default_cfg(epochs=1, batch=4096))
        w = W.aniso(seed=5, ncx=48)
    else:
        wts, w = trained_iso, W.plain_large(seed=3, ncx=64)
    fn = ctx.sweep_aniso if aniso else ctx.sweep
    ctx.set_warmstart(wts, R.DEFAULT_START)
    ref = clone(w.arrays)
    rc, _ = fn(w.model, w.mat, R.FieldSet(ref))                      # the default start, no network
    assert rc == R.MDZ_OK
    try:
        ctx.set_mma_poll_limit(0)
        g = clone(w.arrays)
        rc, st = fn(w.model, w.mat, R.FieldSet(g), flags=R.SWEEP_WARMSTART | R.SWEEP_WARM_TILES, check=False)
    finally:
        ctx.set_mma_poll_limit(-1)
    assert rc == R.MDZ_OK and st.mma_fault == 1
    for k in R.CEN_OUT + R.VER_OUT:
        if ref.get(k) is not None:
            assert np.array_equal(g[k], ref[k], equal_nan=True), k
    # the context works on: a normal warm sweep afterwards
    rc, st = fn(w.model, w.mat, R.FieldSet(clone(w.arrays)), flags=R.SWEEP_WARMSTART | R.SWEEP_WARM_TILES)
    assert rc == R.MDZ_OK and st.mma_fault == 0


def test_warm_start_argument_checks(ctx, trained_iso):
    w = W.plain_small(seed=0, ncx=16)
    ctx.set_warmstart(None)
    rc, _ = ctx.sweep(w.model, w.mat, R.FieldSet(clone(w.arrays)), flags=R.SWEEP_WARMSTART, check=False)
    assert rc == R.MDZ_ENOTREADY
    ctx.set_warmstart(trained_iso, 4)       # 10 features: not the anisotropic network
    wa = W.aniso(seed=4, ncx=16)
    rc, _ = ctx.sweep_aniso(wa.model, wa.mat, R.FieldSet(clone(wa.arrays)), flags=R.SWEEP_WARMSTART, check=False)
    assert rc == R.MDZ_EINVAL
    with pytest.raises(R.RheoError):
        ctx.set_warmstart(trained_iso, 100)


def test_weights_round_trip(tmp_path, trained_iso):
    p = tmp_path / "w.npz"
    trained_iso.save(p)
    w2 = R.MlpWeights.load(p)
    assert bytes(w2) == bytes(trained_iso)
