"""Learned warm start of the local visco-elastic solve: data, training, evaluation.

The reference starts every local Newton solve at the smallest isolated viscosity
(MDLIB/RheologyDensity.c:822-826, AnisotropyRoutines.c:610-612).  This module trains
the small perceptron of csrc/mlp.cuh to predict where the converged viscosity lies
below that start, from pairs that the plain GPU kernel itself produces
(`mdz_rheo_collect`), and measures what the guess saves.  The FP64 Newton iteration
after the guess is unchanged and runs to the same residual tolerance, so the guess
decides only where it starts.

    python -m mdz_warmstart --pairs 8e6 --out warmstart_iso.npz      # collect + train
    python -m mdz_warmstart --eval warmstart_iso.npz                   # iterations saved
"""
import argparse
import json
import math
import time
from typing import Dict, List, Optional, Tuple

import numpy as np

import mdz_rheo as R
import mdz_workloads as W

FEAT_ISO, FEAT_ANISO = 10, 12


def default_cfg(epochs: int = 6, batch: int = 8192, lr: float = 3e-3, seed: int = 7) -> R.MlpTrainCfg:
    return R.MlpTrainCfg(epochs=epochs, batch=batch, lr=lr, lr_final=lr * 0.02, beta1=0.9, beta2=0.999,
                         eps=1e-8, w_pl=0.25, seed=seed)


def collect(ctx: R.Context, workloads, aniso: bool = False, max_pairs: Optional[int] = None
            ) -> Tuple[np.ndarray, np.ndarray]:
    """Run one collecting sweep per workload; keep the items with a finite target."""
    xs, ys, total = [], [], 0
    for w in workloads:
        items = w.mat.Nb_phases * w.nodes
        X = np.empty((items, R.MLP_IN), np.float32)
        Y = np.empty((items, 2), np.float32)
        ctx.collect(w.model, w.mat, R.FieldSet(w.arrays), X, Y, aniso=aniso)
        keep = np.isfinite(Y).all(axis=1)
        xs.append(X[keep])
        ys.append(Y[keep])
        total += int(keep.sum())
        if max_pairs and total >= max_pairs:
            break
    X = np.concatenate(xs)
    Y = np.concatenate(ys)
    if max_pairs and X.shape[0] > max_pairs:
        X, Y = X[:max_pairs], Y[:max_pairs]
    return X, Y


def training_workloads(aniso: bool, pairs: float, seed0: int = 100, ncx: int = 1025):
    """Fresh seeds (never the ones the parity tests or the benchmark use)."""
    need = int(pairs)
    seed = seed0
    while need > 0:
        w = W.aniso(seed=seed, ncx=ncx) if aniso else W.plain_large(seed=seed, ncx=ncx)
        need -= w.mat.Nb_phases * w.nodes
        seed += 1
        yield w


def train(ctx: R.Context, X: np.ndarray, Y: np.ndarray, n_feat: int, cfg: Optional[R.MlpTrainCfg] = None,
          w: Optional[R.MlpWeights] = None):
    cfg = cfg or default_cfg()
    t0 = time.perf_counter()
    w, loss = ctx.train_mlp(X, Y, n_feat, cfg, w)
    return w, loss, time.perf_counter() - t0


def prediction_error(ctx: R.Context, w: R.MlpWeights, X: np.ndarray, Y: np.ndarray) -> Dict[str, float]:
    """Held-out quality of the guess: |z error| quantiles and plastic-flag accuracy."""
    Yp = ctx.mlp_predict(w, X)
    e = np.abs(np.maximum(Yp[:, 0], 0.0) - Y[:, 0])
    acc = float(np.mean((Yp[:, 1] > 0.5) == (Y[:, 1] > 0.5)))
    return {"z_err_median": float(np.median(e)), "z_err_p90": float(np.quantile(e, 0.9)),
            "z_err_p99": float(np.quantile(e, 0.99)), "plastic_accuracy": acc}


def iterations(ctx: R.Context, w: W.Workload, flags: int, aniso: bool = False) -> Dict[str, float]:
    """Mean/max Newton iterations per active (node, phase) of one sweep under `flags`."""
    fn = ctx.sweep_aniso if aniso else ctx.sweep
    a = {k: ([x.copy() for x in v] if isinstance(v, list) else v.copy()) for k, v in w.arrays.items()}
    _, st = fn(w.model, w.mat, R.FieldSet(a), flags=flags)
    return {"mean_iters": st.newton_iters / max(1, st.phase_calls), "max_iters": int(st.max_newton_iters),
            "mean_fp32_steps": st.fp32_steps / max(1, st.phase_calls),
            "phase_calls": int(st.phase_calls), "kernel_ms": float(st.elapsed_ms), "mma_fault": int(st.mma_fault)}


def main(argv: Optional[List[str]] = None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--pairs", type=float, default=8e6)
    ap.add_argument("--ncx", type=int, default=1025)
    ap.add_argument("--aniso", action="store_true")
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--polish", type=int, default=R.DEFAULT_START,
                    help="start descriptor: FP32 Newton steps, plus 256 for the double-float Halley step")
    ap.add_argument("--out", default=None)
    ap.add_argument("--eval", default=None, help="weights file to evaluate instead of training")
    ap.add_argument("--eval-ncx", type=int, default=1025)
    ap.add_argument("--eval-seed", type=int, default=1)
    args = ap.parse_args(argv)
    ctx = R.Context(0)
    n_feat = FEAT_ANISO if args.aniso else FEAT_ISO
    report = {}
    if args.eval:
        wts = R.MlpWeights.load(args.eval)
    else:
        t0 = time.perf_counter()
        X, Y = collect(ctx, training_workloads(args.aniso, args.pairs, ncx=args.ncx), args.aniso, int(args.pairs))
        report["pairs"] = int(X.shape[0])
        report["collect_s"] = time.perf_counter() - t0
        rng = np.random.default_rng(0)
        hold = rng.random(X.shape[0]) < 0.02
        wts, loss, dt = train(ctx, X[~hold], Y[~hold], n_feat,
                              default_cfg(args.epochs, args.batch, args.lr))
        report["train_s"] = dt
        report["loss"] = [float(v) for v in loss]
        report["held_out"] = prediction_error(ctx, wts, X[hold], Y[hold])
        if args.out:
            wts.save(args.out)
    wl = (W.aniso(seed=args.eval_seed, ncx=args.eval_ncx) if args.aniso
          else W.plain_large(seed=args.eval_seed, ncx=args.eval_ncx))
    ctx.set_warmstart(wts, args.polish)
    report["reference_start"] = iterations(ctx, wl, R.SWEEP_REF_START, args.aniso)
    report["default_start"] = iterations(ctx, wl, 0, args.aniso)
    report["warm"] = iterations(ctx, wl, R.SWEEP_WARMSTART, args.aniso)
    report["warm_tiles"] = iterations(ctx, wl, R.SWEEP_WARMSTART | R.SWEEP_WARM_TILES, args.aniso)
    print(json.dumps(report))
    ctx.close()
    return report


if __name__ == "__main__":
    main()
