"""CPU restatement of the warm-start perceptron (test infrastructure only).

The learned warm start has no counterpart in the reference: MDOODZ always starts the
local visco-elastic Newton solve at the smallest isolated viscosity
(MDLIB/RheologyDensity.c:822-826).  The tensor-core training and inference kernels of
the warm start are therefore checked against this float64 numpy statement of the same
network and loss:

    x  = (X - x_shift) * x_scale                       (features >= n_feat are 0)
    a1 = relu(x W1^T + b1),  a2 = relu(a1 W2^T + b2),  o = a2 W3^T + b3
    y0 = (Y0 - z_shift) / z_scale,  y1 = Y1
    L  = (1/n) sum_s [(o0 - y0)^2 + w_pl (o1 - y1)^2]

`bf16=True` rounds every tensor-core operand to bfloat16 (round to nearest even) at
the points where the kernels store BF16 tiles, so that the remaining difference is
only the FP32 accumulation order; `bf16=False` is the exact float64 network.
Only the tests import this module.
"""
import numpy as np

HID, IN = 64, 16


def bf16(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(a, np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    out = u.astype(np.uint32).view(np.float32).astype(np.float64)
    nan = np.isnan(f)
    if nan.any():
        out[nan] = np.nan
    return out


def _q(a, on):
    return bf16(a) if on else np.asarray(a, np.float64)


def weights(w):
    """numpy views of an MlpWeights structure (float64 copies)."""
    d = w.arrays()
    return {k: np.array(v, np.float64) for k, v in d.items()} | {
        "z_shift": float(w.z_shift), "z_scale": float(w.z_scale), "n_feat": int(w.n_feat)}


def normalise(W, X):
    x = (np.asarray(X, np.float32)[:, :IN].astype(np.float32) - W["x_shift"].astype(np.float32)) \
        * W["x_scale"].astype(np.float32)
    x[:, W["n_feat"]:] = 0.0
    return x.astype(np.float64)


def forward(W, X, bf=True):
    x = _q(normalise(W, X), bf)
    a1 = np.maximum(x @ _q(W["W1"], bf).T + W["b1"], 0.0)
    a1q = _q(a1, bf)
    a2 = np.maximum(a1q @ _q(W["W2"], bf).T + W["b2"], 0.0)
    a2q = _q(a2, bf)
    o = a2q @ _q(W["W3"], bf).T + W["b3"]
    return {"x": x, "a1": a1q, "a2": a2q, "o": o}


def predict(W, X, bf=True):
    o = forward(W, X, bf)["o"]
    return np.stack([o[:, 0] * W["z_scale"] + W["z_shift"], o[:, 1]], axis=1)


def gradient(W, X, Y, w_pl=1.0, bf=True):
    """Gradient of L (mean over the n samples) and the summed squared errors."""
    n = X.shape[0]
    f = forward(W, X, bf)
    y0 = (np.asarray(Y[:, 0], np.float32) - np.float32(W["z_shift"])) / np.float32(W["z_scale"])
    e0 = f["o"][:, 0] - y0
    e1 = f["o"][:, 1] - Y[:, 1]
    dy = np.stack([2.0 * e0 / n, 2.0 * w_pl * e1 / n], axis=1)
    dyq = _q(dy, bf)
    g = {"b3": dy.sum(0), "W3": dyq.T @ f["a2"]}
    dz2 = (dyq @ _q(W["W3"], bf)) * (f["a2"] > 0)
    g["b2"] = dz2.sum(0)
    dz2q = _q(dz2, bf)
    g["W2"] = dz2q.T @ f["a1"]
    dz1 = (dz2q @ _q(W["W2"], bf)) * (f["a1"] > 0)
    g["b1"] = dz1.sum(0)
    g["W1"] = _q(dz1, bf).T @ f["x"]
    g["W1"][:, W["n_feat"]:] = 0.0
    loss = np.array([np.sum(e0 * e0), np.sum(w_pl * e1 * e1)])
    return g, loss
