"""The float64 statement of the warm-start network checks itself: its backward pass
against central finite differences of its own loss, and the BF16 rounding helper
against the rounding rule (nearest, ties to even)."""
import numpy as np

import mdz_rheo as R
import mlp_oracle as MO


def make(rng, n_feat=10):
    w = R.MlpWeights()
    w.n_feat = n_feat
    a = w.arrays()
    a["W1"][:, :n_feat] = rng.normal(size=(64, n_feat)) * 0.4
    a["W2"][:] = rng.normal(size=(64, 64)) * 0.2
    a["W3"][:] = rng.normal(size=(2, 64)) * 0.2
    a["b1"][:] = rng.normal(size=64) * 0.1
    a["b2"][:] = rng.normal(size=64) * 0.1
    a["b3"][:] = rng.normal(size=2) * 0.1
    a["x_scale"][:n_feat] = 1.0
    w.z_shift, w.z_scale = 0.5, 2.0
    return w


def loss_of(Wd, X, Y, w_pl):
    o = MO.forward(Wd, X, bf=False)["o"]
    y0 = (Y[:, 0].astype(np.float32) - np.float32(Wd["z_shift"])) / np.float32(Wd["z_scale"])
    return np.mean((o[:, 0] - y0) ** 2 + w_pl * (o[:, 1] - Y[:, 1]) ** 2)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    n = 64
    X = np.zeros((n, 16), np.float32)
    X[:, :10] = rng.normal(size=(n, 10))
    Y = rng.normal(size=(n, 2)).astype(np.float32)
    Wd = MO.weights(make(rng))
    g, _ = MO.gradient(Wd, X, Y, 0.7, bf=False)
    h = 1e-6
    for k, idx in [("W1", (3, 4)), ("W1", (60, 9)), ("b1", (5,)), ("W2", (7, 11)), ("b2", (63,)),
                   ("W3", (1, 30)), ("W3", (0, 2)), ("b3", (0,)), ("b3", (1,))]:
        P = {kk: (v.copy() if isinstance(v, np.ndarray) else v) for kk, v in Wd.items()}
        M = {kk: (v.copy() if isinstance(v, np.ndarray) else v) for kk, v in Wd.items()}
        P[k][idx] += h
        M[k][idx] -= h
        fd = (loss_of(P, X, Y, 0.7) - loss_of(M, X, Y, 0.7)) / (2 * h)
        assert abs(fd - g[k][idx]) <= 1e-6 * max(1.0, abs(fd)), (k, idx, fd, g[k][idx])


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -9, -2.5, 3.0e38, 1e-40], np.float32)
    r = MO.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                            # 1 + 2^-8 is the tie between 1 and 1 + 2^-7
    assert r[2] == 1.0 + 2 ** -7                  # above the tie
    assert r[3] == 1.0
    assert r[4] == -2.5
    assert np.isfinite(r[5])
    assert MO.bf16(np.array([np.nan], np.float32))[0] != MO.bf16(np.array([np.nan], np.float32))[0]
