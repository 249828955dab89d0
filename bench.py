#!/usr/bin/env python
"""Benchmark of the GB300 local rheology update (MDOODZ7.0 NonNewtonianViscosityGrid).

Metric: rheology point-updates/s on 1 GB300 (FP64 local solves to the reference's
residual tolerance; the learned warm start and the reference's own start point are
timed beside the default path).  A point-update is one
centroid or vertex fully processed by the sweep: every active phase's local solve,
phase averaging and the final stress.  One step = one sweep over the 2049 x 2049-cell,
5-phase grid (4,198,401 centroids + 4,202,500 vertices), synthetic seeded inputs.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--no-warm]

Timed forms of the same sweep (all iterate each local FP64 Newton solve to
|r| < 1e-13 Eii, the reference's criterion):
  value            default start: up to 4 FP32 Newton steps from the reference's start
                   point, then one Halley step evaluated in double-float
  reference_start  the reference's own start point (eta_up), its iteration counts
  warm_start       learned warm start: the network's guess (BF16 tensor-core MMAs per warp)
                   before the same start stages; the network is trained here first, on
                   pairs collected by the plain kernel from a fresh seed (1025 x 1025
                   cells, 8M pairs); the line also carries its ablations
The default line adds the anisotropic 4097^2 sweep and the 64-grid batch (--no-configs
skips them), the Newton operator, StrainRateComponents, the input preparation and
UpdateParticleStress.

`value` is timed with CUDA events on the launching stream with inputs resident in
HBM (3.3 GB of fields, larger than the 129 MB L2, so no flush between steps);
`e2e` is the same sweep through the C ABI on page-locked host arrays, which the kernels
read and write over the coherent host link inside the timed region (no staging copies);
the line also carries the staged forms (host<->device copies in row bands, and in one
piece) and the same calls on ordinary pageable arrays (read in place where the GPU reads
pageable memory through the host page tables).  Under torchrun each rank sweeps its own grid
(independent instances, weak scaling; the path has no exchange step).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "mdoodz7.0_gb300"))

REP_SEED_HEADLINE = 1  # the headline grid's seed (rank 0)
METRIC = "rheology point-updates/s on 1 GB300: plain FP64 vs NN warm-start at tol 1e-11"
UNIT = "point-updates/s"

# FP64 work of the sweep per point-update, in flops (DFMA = 2, DADD/DMUL = 1): ncu's
# thread-level FP64 instruction counters of one sweep's two launches (centroids, then
# vertices; default start, default form: k_sweep_compact for the isotropic sweep, k_sweep
# for the anisotropic one), summed, on the same field distributions at 513 x 513 cells
# (527,365 nodes), per workload (profiles/k_sweep_plain_large_513.md,
# profiles/k_sweep_aniso_513.md).  `roofline.achieved` = this x nodes / the CUDA-event
# time of one sweep (events before the first launch and after the second).
FP64_FLOPS_PER_POINT = {"plain_large": 1448.7, "aniso": 1038.4}
# FP64 work of the batched many-grid sweep per local solve (phase call), same convention:
# the two k_sweep_batch launches of one sweep of an 8-grid batch of the many-grid
# distribution (5,096,155 phase calls; profiles/k_sweep_batch_many_grids.md); the grids
# have 2 to 5 phases, so the work is counted per phase call.
FP64_FLOPS_PER_PHASE_CALL = {"many_grids": 288.8}
# DRAM bytes (read + write) per point-update of one sweep's two launches at 1025 x 1025
# cells (0.7 GB of fields, five times L2; profiles/k_sweep_spills_and_dram_1025.md: the
# default forms at 4 CTAs per SM, whose register spills reach DRAM in part), scaled to a
# sweep by its node count.
DRAM_BYTES_PER_POINT = {"plain_large": 414.6, "aniso": 364.2}
# FP64 work of k_marker_update per marker (inactive ones included), same convention:
# thread-level counters of one launch at 513 x 513 cells with 16 markers per cell
# (4,210,704 markers) per option set (profiles/k_marker_update_513.md).
FP64_FLOPS_PER_MARKER = {"jaumann_stencil1": 90.48, "analytical_director_stencil9": 218.31}
# FP64 work of the Newton operator per perturbed local solve, same convention: one launch of
# k_operators_compact at 513 x 513 cells (21,094,600 perturbed solves;
# profiles/k_operators_newton_257.md).
FP64_FLOPS_PER_OPERATOR_SOLVE = 224.7
# FP64-pipe thread instructions (DFMA, DADD, DMUL and the few conversions; each takes a
# pipe slot whether it carries two flops or one) per unit, from the same captures:
# `fp64_issue_frac` = this x units / time / (measured DFMA rate / 2) is how busy the FP64
# pipe is with useful lanes, the figure the flop fraction understates by the DADD/DMUL share.
FP64_THREAD_INSTS = {"plain_large": 954.4, "aniso": 671.0, "many_grids": 190.0,
                     "jaumann_stencil1": 77.23, "analytical_director_stencil9": 183.50,
                     "newton_operator": 148.7}


def issue_frac(insts_per_unit, units, ms, peak_tflops):
    """FP64-pipe thread instructions per second over the DFMA lane rate (peak flops / 2)."""
    if not insts_per_unit or not ms:
        return None
    return insts_per_unit * units / (ms * 1e-3) / (peak_tflops * 1e12 / 2.0)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=None,
                    help="cells per side (default 2049; 4097 for --workload aniso)")
    ap.add_argument("--workload", default="plain_large", choices=["plain_large", "aniso", "many_grids"],
                    help="plain_large: the headline; aniso: ViscosityConciseAniso sweep; many_grids: "
                         "64 uneven grids in one launch and a 20-sweep CUDA graph")
    ap.add_argument("--phases", type=int, default=5)
    ap.add_argument("--grids", type=int, default=64, help="grids of the many-grid workload")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-warm", action="store_true", help="skip the learned warm start")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--no-operators", action="store_true", help="skip the Newton-operator timing")
    ap.add_argument("--no-strain-rates", action="store_true", help="skip the StrainRateComponents timing")
    ap.add_argument("--no-prep", action="store_true", help="skip the Softening / ShearModCompExpGrid timing")
    ap.add_argument("--no-markers", action="store_true", help="skip the UpdateParticleStress timing")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the anisotropic 4097^2 and the 64-grid sections of the default line")
    args = ap.parse_args()
    if args.size is None:
        args.size = 4097 if args.workload == "aniso" else 2049
    if args.workload == "aniso" and args.phases == 5:
        args.phases = 3
    return args


def dist_env():
    import mdz_replicas
    return mdz_replicas.dist_env()


def algorithmic_bytes(w, aniso=False):
    """Compulsory HBM bytes of one sweep: every input field read once, every output
    written once (field counts of NonNewtonianViscosityGrid, RheologyDensity.c:1131-1426;
    the anisotropic sweep adds d1, d2, angle and the anisotropy factor, and VE_s)."""
    np_ = w.mat.Nb_phases
    nc, nv = w.Nc, w.Nv
    extra_in = 4 if aniso else 0
    cen = 8 * (18 + extra_in + np_ + np_) + 1 + 8 * 23                  # inputs, fractions, phase_eta, BC, outputs
    ver = 8 * (13 + extra_in + np_ + np_) + 1 + 8 * (6 + int(aniso)) + 8 * 4   # + the four interpolated fields
    return nc * cen + nv * ver


def strain_rate_bytes(nx, nz):
    """Compulsory HBM bytes of one StrainRateComponents launch (RheologyDensity.c:2001-2097)
    on a grid without air: u_in (Nx*(Nz+1)) and v_in ((Nx+1)*Nz) read, BCp and BCg read
    (1 byte each), five centroid and five vertex fields written once."""
    nc, nv = (nx - 1) * (nz - 1), nx * nz
    return 8 * (nx * (nz + 1) + (nx + 1) * nz) + nc + nv + 8 * 5 * (nc + nv)


def prep_bytes(step, nc, nv, nphases):
    """Compulsory HBM bytes of one preparation launch on a grid without air: every phase
    fraction and BC flag read once; softening also reads the plastic strain and the noise
    (8 + 8 B) and writes fric, dil, C (24 B) per node; the shear modulus writes mu, bet,
    alp at centroids (24 B) and mu, bet at vertices (16 B)."""
    reads = (nc + nv) * (8 * nphases + 1)
    if step == "softening":
        return reads + (nc + nv) * (16 + 24)
    return reads + nc * 24 + nv * 16


def marker_bytes(n, nx, nz, director):
    """Compulsory HBM bytes of one UpdateParticleStress call (RheologyParticles.c:1725-2004)
    on a grid without air: per marker x, z and phase read (20 B) and its three stresses
    read and written (48 B), with the director its two components read and written
    (32 B); the grid's new and old centroid stresses (32 B) and BCp read once, the new
    and old vertex shear stress (16 B) and BCg read and wxz read and written (16 B), and
    with the director u_in and v_in read.  The vertex weight-sum scratch is not counted."""
    nc, nv = (nx - 1) * (nz - 1), nx * nz
    b = n * (20 + 48 + (32 if director else 0)) + nc * 33 + nv * 33
    if director:
        b += 8 * (nx * (nz + 1) + (nx + 1) * nz)
    return b


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="mdz_clocks_", suffix=".csv")
        os.close(fd)

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.2)
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower() == "active"})
        try:
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": reasons}


def cpu_baseline(W, O, sample_cells=1025, reps=1, aniso=False):
    """The oracle (C restatement of the reference, OpenMP, all host cores) on a bounded
    sample of the same workload distribution."""
    import mdz_rheo as R
    ws = W.aniso(seed=101, ncx=sample_cells) if aniso else W.plain_large(seed=101, ncx=sample_cells)
    O.orc_sweep(ws.model, ws.mat, R.FieldSet(ws.arrays), aniso=aniso)  # warm-up (page faults, threads)
    t0 = time.perf_counter()
    for _ in range(reps):
        O.orc_sweep(ws.model, ws.mat, R.FieldSet(ws.arrays), aniso=aniso)
    dt = (time.perf_counter() - t0) / reps
    lib = O.reference()
    kind = "port"
    return {"value": ws.nodes / dt, "unit": UNIT, "cores": O.oracle().orc_num_threads(), "kind": kind,
            "sample": f"{sample_cells}x{sample_cells}-cell grid of the same {ws.mat.Nb_phases}-phase workload "
                      f"({ws.nodes} nodes), {reps} sweep(s), {dt:.2f} s each"}


def marker_cpu_baseline(W, O, sample_cells=1025):
    """UpdateParticleStress on the oracle (the C restatement, one thread) on a bounded
    sample of the marker workload, Jaumann rotation and the 1-cell stencil."""
    import mdz_rheo as R
    mw = W.marker_workload(seed=103, ncx=sample_cells, markers_per_cell=16)
    opts = R.MarkerOpts()
    opts.elastic, opts.stress_rotation, opts.anisotropy, opts.advection, opts.interp_stencil = 1, 1, 0, 1, 1
    grid = {k: v.copy() for k, v in mw.arrays.items()}
    mk = {k: v.copy() for k, v in mw.info["markers"].items()}
    t0 = time.perf_counter()
    O.orc_marker_stress(mw.model, opts, grid, mk, mw.info["dx"], mw.info["dz"])
    dt = time.perf_counter() - t0
    n = int(mk["x"].size)
    return {"value": n / dt, "unit": "markers/s", "cores": 1, "kind": "port",
            "sample": f"{sample_cells}x{sample_cells} cells, 16 markers per cell ({n} markers), one call, "
                      f"{dt:.2f} s"}


def run_reference(args):
    """--impl reference: the reference's own NonNewtonianViscosityGrid, compiled from the
    MDOODZ7.0 sources by oracle/Makefile with the reference's release flags (on a host
    without the tree, from the preprocessed units the build wrote beside it), timed on
    all host cores (OpenMP) on the same 2049 x 2049, 5-phase workload as our line.  Only
    where neither exists does the C restatement of the same code (bit-identical, pinned
    by the tests) stand in, and the line says so (kind "port")."""
    ws_, rank, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import mdz_rheo as R
    import mdz_workloads as W
    import oracle_lib as O
    O.build(ref=True)
    sample = args.size
    w = W.plain_large(seed=REP_SEED_HEADLINE, ncx=sample, nphases=args.phases)
    ref = O.reference()
    kind = "reference" if ref is not None else "port"

    def step():
        fs = R.FieldSet(w.arrays)
        if ref is not None:
            O.ref_sweep(w.model, w.mat, fs)
        else:
            O.orc_sweep(w.model, w.mat, fs)

    for _ in range(args.warmup):
        step()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    ms = 1e3 * statistics.mean(times)
    value = w.nodes / (ms * 1e-3)
    cores = O.oracle().orc_num_threads()
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"plain_large: {args.size}x{args.size} cells, {args.phases} phases (dislocation, "
                                   "diffusion, Peierls, softened Drucker-Prager); the reference's own local Newton "
                                   "to |r| < 1e-13 Eii from its own start",
                       "nodes_per_step": w.nodes, "same_config": True,
                       "what": ("NonNewtonianViscosityGrid of MDOODZ7.0 (RheologyDensity.c:1131), compiled from its "
                                "sources with -O3 -ftree-vectorize -funroll-loops -fopenmp -D_OMP_")
                               if ref is not None else "the C restatement of NonNewtonianViscosityGrid"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": f"the whole {sample}x{sample}-cell grid, {w.nodes} nodes per step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_many_grids(args):
    """--workload many_grids: the 64-grid workload alone (many_grids_section), its graph of
    20 batched sweeps with the default start as the line's value."""
    import torch

    import mdz_replicas as REP
    import mdz_rheo as R

    ws, rank, local = dist_env()
    if ws > 1:
        torch.cuda.set_device(local)
        REP.init("nccl")
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    ctx = R.Context(dev)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    with ClockSampler(dev) as clk:
        mg, _ = many_grids_section(args, ctx, dev, ws, rank, stream, barrier)
    if rank != 0:
        REP.finalize()
        return
    g = mg["graph"]["default"]
    line = {"metric": METRIC, "value": g["value"], "unit": UNIT, "n_gpus": ws, "steps": max(1, args.steps // 4),
            "warmup": args.warmup, "ms_per_step": g["ms_per_graph"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": mg["workload"], "nodes_per_sweep": mg["nodes_per_sweep"],
                       "sweeps_per_step": mg["sweeps_per_graph"], "l2": "inputs larger than L2, no flush"},
            "forms_ms_per_sweep": mg["forms_ms_per_sweep"], "graph": mg["graph"],
            "roofline": None, "cpu_baseline": None, "e2e": None, "clocks": clk.summary(),
            "gpu_launches": max(1, args.steps // 4) * g["kernel_launches_per_graph"]}
    print(json.dumps(line))
    if ws > 1:
        REP.finalize()


def timed_sweeps(args, fn, w, fs, flags, stream, barrier, dev, reps=None):
    """W warm-up sweeps, then `reps` (default K) timed between barriers, CUDA events on the
    context's stream; returns (ms per sweep, max over ranks; the last sweep's statistics)."""
    import torch

    import mdz_replicas as REP
    import mdz_rheo as R
    reps = reps or args.steps
    for _ in range(args.warmup):
        fn(w.model, w.mat, fs, mem=R.MEM_DEVICE, flags=flags)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(stream)
    stats = []
    for _ in range(reps):
        _, st = fn(w.model, w.mat, fs, mem=R.MEM_DEVICE, flags=flags)
        stats.append(st)
    e1.record(stream)
    barrier()
    return REP.max_over_ranks(e0.elapsed_time(e1), dev) / reps, stats


def sweep_summary(ms, stats, nodes, ws):
    import mdz_replicas as REP
    calls = max(1, sum(int(x.phase_calls) for x in stats))
    return {"value": REP.whole_job_rate(nodes, ws, ms), "unit": UNIT, "ms_per_step": ms,
            "mean_newton_iters": sum(int(x.newton_iters) for x in stats) / calls,
            "max_newton_iters": max(int(x.max_newton_iters) for x in stats),
            "mean_fp32_steps": sum(int(x.fp32_steps) for x in stats) / calls,
            "kernel_ms_per_sweep": statistics.mean(x.elapsed_ms for x in stats)}


def aniso_section(args, ctx, dev, ws, rank, stream, barrier, no_warm):
    """The anisotropic workload: ViscosityConciseAniso over 4097 x 4097 cells, 3 phases,
    on the device; the default start, the reference's start and the learned warm start (a
    12-input network trained here on pairs the plain kernel produces from a fresh seed),
    and end to end through the C ABI with page-locked host buffers."""
    import torch

    import mdz_replicas as REP
    import mdz_rheo as R
    import mdz_workloads as W
    t0 = time.perf_counter()
    w = W.aniso(seed=REP.replica_seed(4, rank), ncx=4097, nphases=3)
    gen_s = time.perf_counter() - t0
    d = {k: ([torch.from_numpy(x).to(dev) for x in v] if isinstance(v, list) else torch.from_numpy(v).to(dev))
         for k, v in w.arrays.items()}
    fs = R.FieldSet(d)
    fn = ctx.sweep_aniso
    tune = None
    if not args.no_autotune:  # each start keeps its own choice (the reference's: 10 bisection steps, Newton)
        tune = {"candidates": list(R.Context.AUTOTUNE_NAMES)}
        for label, fl in (("default_start", 0), ("reference_start", R.SWEEP_REF_START)):
            t_ms, t_best, t_shape = ctx.autotune(w.model, w.mat, fs, aniso=True, flags=fl, reps=1)
            tune[label] = {"ms_per_sweep": [float(x) for x in t_ms], "chosen": int(t_best),
                           "block": t_shape[0], "grid_cap": t_shape[1], "form": ctx.launch_form(True)}
    ms, st = timed_sweeps(args, fn, w, fs, 0, stream, barrier, dev)
    out = sweep_summary(ms, st, w.nodes, ws)
    out["autotune"] = tune
    out.update({"workload": "aniso: 4097x4097 cells, 3 phases (dislocation, softened Drucker-Prager), director "
                            "angle U[0,pi), anisotropy factor log-U(1,10); FP64 local Newton to |r| < 1e-13 Eii",
                "nodes": w.nodes, "generate_s": gen_s,
                "algorithmic_bytes_per_sweep": algorithmic_bytes(w, True)})
    ms_r, st_r = timed_sweeps(args, fn, w, fs, R.SWEEP_REF_START, stream, barrier, dev)
    out["reference_start"] = sweep_summary(ms_r, st_r, w.nodes, ws)
    if not no_warm:
        import mdz_warmstart as WSt
        src = W.aniso(seed=130 + 1000 * rank, ncx=1449, nphases=3)
        Xs, Ys = WSt.collect(ctx, [src], aniso=True, max_pairs=8_000_000)
        del src
        wts, loss, train_s = WSt.train(ctx, Xs, Ys, WSt.FEAT_ANISO)
        del Xs, Ys
        ctx.set_warmstart(wts, R.DEFAULT_START)
        ms_w, st_w = timed_sweeps(args, fn, w, fs, R.SWEEP_WARMSTART, stream, barrier, dev)
        ctx.set_warmstart(None, R.DEFAULT_START)
        out["warm_start"] = sweep_summary(ms_w, st_w, w.nodes, ws)
        out["warm_start"].update({"train_s": train_s, "final_train_loss": float(loss[-1])})
    if not args.no_e2e:
        h = {k: ([torch.from_numpy(x).pin_memory() for x in v] if isinstance(v, list)
                 else torch.from_numpy(v).pin_memory()) for k, v in w.arrays.items()}
        fh = R.FieldSet(h)
        for _ in range(max(1, args.warmup)):
            fn(w.model, w.mat, fh, mem=R.MEM_HOST)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            _, est = fn(w.model, w.mat, fh, mem=R.MEM_HOST)
        e1.record(stream)
        barrier()
        e2e_ms = REP.max_over_ranks(e0.elapsed_time(e1) / args.steps, dev)
        out["e2e"] = {"value": REP.whole_job_rate(w.nodes, ws, e2e_ms), "unit": UNIT, "ms_per_step": e2e_ms,
                      "h2d_bytes_per_step": int(est.h2d_bytes), "d2h_bytes_per_step": int(est.d2h_bytes)}
        del h, fh
    del d, fs, w
    torch.cuda.empty_cache()
    return out


def many_grid_network(ctx, rank):
    """The 10-input network for the many-grid workload, trained on pairs the plain kernel
    produces on a separate batch of the same distribution (fresh seed): its time steps
    (1e10-1e12 s) and phase counts are not the single grid's."""
    import mdz_rheo as R
    import mdz_warmstart as WSt
    import mdz_workloads as W
    src = W.many_grids(seed=700 + 1000 * rank, n=24)
    Xs, Ys = WSt.collect(ctx, src, max_pairs=8_000_000)
    del src
    wts, loss, train_s = WSt.train(ctx, Xs, Ys, WSt.FEAT_ISO)
    return wts, {"pairs": int(Xs.shape[0]), "train_s": train_s, "final_train_loss": float(loss[-1])}


def many_grids_section(args, ctx, dev, ws, rank, stream, barrier, warm=False):
    """The many-grid workload: 64 grids of uneven size (65-1025 cells per side, 2-5 phases,
    dt 1e10-1e12 s, each with its own seed), device-resident.  Forms of one Picard sweep
    over all of them:
    64 separate sweep calls, one batched sweep (two launches), and a CUDA graph of 20
    batched sweeps with the strain rates perturbed by +-5 % in each (fused into the
    sweep's load), with the default start and (warm) with the learned warm start, its
    network trained on a separate batch of the same distribution."""
    import torch

    import mdz_replicas as REP
    import mdz_rheo as R
    import mdz_workloads as W
    t0 = time.perf_counter()
    grids = W.many_grids(seed=REP.replica_seed(7, rank), n=args.grids)
    gen_s = time.perf_counter() - t0
    devs = [{k: ([torch.from_numpy(x).to(dev) for x in v] if isinstance(v, list) else torch.from_numpy(v).to(dev))
             for k, v in g.arrays.items()} for g in grids]
    fss = [R.FieldSet(d) for d in devs]
    nodes = sum(g.nodes for g in grids)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(step, reps):
        for _ in range(args.warmup):
            step()
        barrier()
        e0.record(stream)
        for _ in range(reps):
            step()
        e1.record(stream)
        barrier()
        return REP.max_over_ranks(e0.elapsed_time(e1), dev) / reps

    def separate():
        for g, fs in zip(grids, fss):
            ctx.sweep(g.model, g.mat, fs, mem=R.MEM_DEVICE)

    ms_sep = timed(separate, args.steps)
    # The captured sweeps perturb the strain rates in place, each sweep from the previous
    # one's (a Picard loop within one time step).  Every graph launch is one time step: it
    # starts from the step's strain rates, copied back on the stream before the launch
    # (inside the timed region), so repeated launches do not random-walk the inputs away
    # from the workload's distribution.
    rates = ("exxd", "ezzd", "exz_n", "exxd_s", "ezzd_s", "exz")
    saved = [{k: d[k].clone() for k in rates} for d in devs]

    def restore():
        for d, s in zip(devs, saved):
            for k in rates:
                d[k].copy_(s[k])

    nsw, amp = 20, 0.05
    forms = {"separate_calls": ms_sep}
    graphs = {}
    wts, train = (many_grid_network(ctx, rank) if warm else (None, None))
    for label, flags in (("default", 0), ("warm", R.SWEEP_WARMSTART)):
        if flags and wts is None:
            continue
        if flags:
            ctx.set_warmstart(wts, R.DEFAULT_START)
        batch = R.Batch(ctx, [g.model for g in grids], [g.mat for g in grids], fss, flags=flags)
        calls = [0]

        def batched():
            _, st = batch.sweep()
            calls[0] = st.phase_calls

        forms[f"one_batched_launch_{label}"] = timed(batched, args.steps)
        # the same launch as a persistent grid: 3 resident CTAs per SM striding over the tiles
        batch.set_grid(3 * torch.cuda.get_device_properties(dev).multi_processor_count)
        forms[f"one_batched_launch_{label}_persistent_grid"] = timed(batched, args.steps)
        batch.set_grid(0)
        batch.capture(nsw, amp=amp, seed=2026)
        stats = []

        def graph():
            restore()
            _, st = batch.launch()
            stats.append(st)

        ms_graph = timed(graph, max(1, args.steps // 4))
        restore()
        forms[f"graph_{label}"] = ms_graph / nsw
        st = stats[-1]
        graphs[label] = {"value": REP.whole_job_rate(nodes * nsw, ws, ms_graph), "unit": UNIT,
                         "ms_per_graph": ms_graph, "ms_per_sweep": ms_graph / nsw,
                         "phase_calls_per_sweep": int(calls[0]),
                         "mean_newton_iters": st.newton_iters / max(1, st.phase_calls),
                         "max_newton_iters": int(st.max_newton_iters),
                         "mean_fp32_steps": st.fp32_steps / max(1, st.phase_calls),
                         "kernel_launches_per_graph": int(st.kernel_launches)}
        batch.close()
        if flags:
            ctx.set_warmstart(None, R.DEFAULT_START)
    sides = sorted(g.model.Nx - 1 for g in grids)
    out = {"workload": f"many_grids: {len(grids)} grids, {sides[0]}-{sides[-1]} cells per side (log-uniform), 2-5 phases "
                       "each, dt 1e10-1e12 s; one CUDA graph of 20 batched sweeps, strain rates x (1 + 0.05 "
                       "U[-1,1)) in each (fused into the sweep's load), every launch from the time step's "
                       "strain rates (copied back before it, inside the timed region)",
           "nodes_per_sweep": nodes, "sweeps_per_graph": nsw, "generate_s": gen_s,
           "value": graphs["default"]["value"], "unit": UNIT, "ms_per_sweep": graphs["default"]["ms_per_sweep"],
           "graph": graphs, "forms_ms_per_sweep": forms, "warm_network": train,
           "separate_vs_graph": ms_sep / graphs["default"]["ms_per_sweep"]}
    del devs, fss, saved
    torch.cuda.empty_cache()
    return out, grids[:4]


def many_grids_cpu_baseline(O, grids):
    """The oracle (C restatement, OpenMP on the host cores) on a few grids of the same batch."""
    import mdz_rheo as R
    nodes = sum(g.nodes for g in grids)
    for g in grids[:1]:
        O.orc_sweep(g.model, g.mat, R.FieldSet(g.arrays))
    t0 = time.perf_counter()
    for g in grids:
        O.orc_sweep(g.model, g.mat, R.FieldSet(g.arrays))
    dt = time.perf_counter() - t0
    sides = ", ".join(str(g.model.Nx - 1) for g in grids)
    return {"value": nodes / dt, "unit": UNIT, "cores": O.oracle().orc_num_threads(), "kind": "port",
            "sample": f"the batch's first {len(grids)} grids ({sides} cells per side, {nodes} nodes), one sweep "
                      f"each, {dt:.2f} s"}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "many_grids":
        run_many_grids(args)
        return
    import numpy as np
    import torch

    import mdz_rheo as R
    import mdz_workloads as W

    import mdz_replicas as REP
    ws, rank, local = dist_env()
    if ws > 1:
        torch.cuda.set_device(local)
        REP.init("nccl")
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)

    aniso = args.workload == "aniso"
    if aniso:
        w = W.aniso(seed=REP.replica_seed(4, rank), ncx=args.size, nphases=args.phases)
    else:
        w = W.plain_large(seed=REP.replica_seed(1, rank), ncx=args.size, nphases=args.phases)
    d = {k: ([torch.from_numpy(x).to(dev) for x in v] if isinstance(v, list) else torch.from_numpy(v).to(dev))
         for k, v in w.arrays.items()}
    fs = R.FieldSet(d)
    ctx = R.Context(dev)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    sweep = ctx.sweep_aniso if aniso else ctx.sweep
    tune = None
    if not args.no_autotune:  # launch shape for this grid, before any timed region
        # every candidate form, from the default start and from the reference's start (where
        # the local Newton's iteration counts are most uneven: 1 to 8); each start keeps its
        # own choice
        tune = {"candidates": list(R.Context.AUTOTUNE_NAMES)}
        for label, fl in (("default_start", 0), ("reference_start", R.SWEEP_REF_START)):
            t_ms, t_best, t_shape = ctx.autotune(w.model, w.mat, fs, aniso=aniso, flags=fl, reps=2)
            tune[label] = {"ms_per_sweep": [float(x) for x in t_ms], "chosen": int(t_best),
                           "block": t_shape[0], "grid_cap": t_shape[1], "form": ctx.launch_form(aniso)}

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def timed(flags, clock=False):
        """Device-resident sweeps: W warm-up, then K timed between barriers (max over ranks)."""
        for _ in range(args.warmup):
            sweep(w.model, w.mat, fs, mem=R.MEM_DEVICE, flags=flags)
        r = {"kernel_ms": [], "iters": 0, "calls": 0, "launches": 0, "maxit": 0, "f32": 0, "fault": 0}
        barrier()
        clk = ClockSampler(dev) if clock else None
        if clk:
            clk.__enter__()
        e0.record(stream)
        for _ in range(args.steps):
            rc, st = sweep(w.model, w.mat, fs, mem=R.MEM_DEVICE, flags=flags)
            r["kernel_ms"].append(st.elapsed_ms)
            r["iters"] += st.newton_iters
            r["calls"] += st.phase_calls
            r["launches"] += st.kernel_launches
            r["maxit"] = max(r["maxit"], st.max_newton_iters)
            r["f32"] += st.fp32_steps
            r["fault"] |= st.mma_fault
        e1.record(stream)
        barrier()
        if clk:
            clk.__exit__()
            r["clocks"] = clk.summary()
        total_ms = REP.max_over_ranks(e0.elapsed_time(e1), dev)
        r["ms_step"] = total_ms / args.steps
        r["value"] = REP.whole_job_rate(w.nodes, ws, r["ms_step"])
        r["mean_iters"] = r["iters"] / max(r["calls"], 1)
        r["mean_f32"] = r["f32"] / max(r["calls"], 1)
        return r

    def summary(r):
        return {"value": r["value"], "unit": UNIT, "ms_per_step": r["ms_step"],
                "mean_newton_iters": r["mean_iters"], "max_newton_iters": r["maxit"],
                "mean_fp32_steps": r["mean_f32"], "kernel_ms_per_sweep": statistics.mean(r["kernel_ms"])}

    # ---- the default path: the headline ----
    main_r = timed(0, clock=True)
    kernel_ms, launches, calls = main_r["kernel_ms"], main_r["launches"], main_r["calls"]
    ms_step, value, clk_summary = main_r["ms_step"], main_r["value"], main_r["clocks"]
    # ---- end to end through the C ABI with pinned host buffers, on the headline grid before
    # the other timings fill host memory ----
    e2e = None
    if not args.no_e2e:
        h = {k: ([torch.from_numpy(x).pin_memory() for x in v] if isinstance(v, list)
                 else torch.from_numpy(v).pin_memory()) for k, v in w.arrays.items()}
        fh = R.FieldSet(h)
        for _ in range(max(1, args.warmup)):
            sweep(w.model, w.mat, fh, mem=R.MEM_HOST)
        barrier()
        e0.record(stream)
        bi = bo = 0
        for _ in range(args.steps):
            rc, st = sweep(w.model, w.mat, fh, mem=R.MEM_HOST)
            bi, bo = st.h2d_bytes, st.d2h_bytes
        e1.record(stream)
        barrier()
        e2e_ms = REP.max_over_ranks(e0.elapsed_time(e1) / args.steps, dev)
        direct = st.kernel_launches == 2  # the kernels addressed the page-locked arrays in place

        def staged(bands):
            """The same calls with every array staged through device copies (MDZ_SWEEP_STAGED)."""
            ctx.set_host_bands(bands)
            sweep(w.model, w.mat, fh, mem=R.MEM_HOST, flags=R.SWEEP_STAGED)
            barrier()
            e0.record(stream)
            for _ in range(args.steps):
                _, sst = sweep(w.model, w.mat, fh, mem=R.MEM_HOST, flags=R.SWEEP_STAGED)
            e1.record(stream)
            barrier()
            ctx.set_host_bands(0)
            ms = REP.max_over_ranks(e0.elapsed_time(e1) / args.steps, dev)
            # a vertex kernel per band, a centroid kernel per band with centroid rows
            return {"value": REP.whole_job_rate(w.nodes, ws, ms), "ms_per_step": ms,
                    "row_bands": int((sst.kernel_launches + 1) // 2)}

        e2e = {"value": REP.whole_job_rate(w.nodes, ws, e2e_ms), "unit": UNIT, "ms_per_step": e2e_ms,
               "h2d_bytes_per_step": int(bi), "d2h_bytes_per_step": int(bo),
               "how": ("mdz_rheo_sweep on page-locked host arrays, which the kernels read and write in "
                       "place over the coherent host link: the inputs cross to the device and the outputs "
                       "back inside the timed region, with no staging copies" if direct else
                       "mdz_rheo_sweep on host arrays staged through device copies in row bands"),
               "staged_row_bands": staged(0),
               "staged_one_band": staged(1)}
        del h, fh
        # the same calls on ordinary pageable host arrays, as a simulation code allocates them
        pg = {k: ([x.copy() for x in v] if isinstance(v, list) else v.copy()) for k, v in w.arrays.items()}
        fpg = R.FieldSet(pg)
        sweep(w.model, w.mat, fpg, mem=R.MEM_HOST)
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            _, pst = sweep(w.model, w.mat, fpg, mem=R.MEM_HOST)
        e1.record(stream)
        barrier()
        pg_ms = REP.max_over_ranks(e0.elapsed_time(e1) / args.steps, dev)
        e2e["pageable_arrays"] = {"value": REP.whole_job_rate(w.nodes, ws, pg_ms), "ms_per_step": pg_ms,
                                  "in_place": bool(ctx.pageable_in_place()),
                                  "kernel_launches_per_step": int(pst.kernel_launches)}
        del pg, fpg

    # ---- the reference's own start point (same kernel, same tolerance) ----
    ref_r = summary(timed(R.SWEEP_REF_START))
    # ---- the FP32 Newton steps without the double-float Halley step ----
    ctx.set_warmstart(None, R.DEFAULT_POLISH)
    fp32_r = summary(timed(0))
    ctx.set_warmstart(None, R.DEFAULT_START)
    # ---- learned warm start ----
    warm = None
    wts = None
    if not args.no_warm:
        import mdz_warmstart as WSt
        t0 = time.perf_counter()
        if aniso:
            src = W.aniso(seed=130 + 1000 * rank, ncx=1449, nphases=args.phases)
        else:
            src = W.plain_large(seed=100 + 1000 * rank, ncx=1025, nphases=args.phases)
        Xs, Ys = WSt.collect(ctx, [src], aniso=aniso, max_pairs=8_000_000)
        del src
        t1 = time.perf_counter()
        wts, loss, train_s = WSt.train(ctx, Xs, Ys, WSt.FEAT_ANISO if aniso else WSt.FEAT_ISO)
        del Xs, Ys
        ctx.set_warmstart(wts, R.DEFAULT_START)
        warm = summary(timed(R.SWEEP_WARMSTART))
        tiles = timed(R.SWEEP_WARMSTART | R.SWEEP_WARM_TILES)
        tiles_s = summary(tiles)
        tiles_s["mma_fault"] = int(tiles["fault"])
        ctx.set_warmstart(wts, R.START_DD)  # the network's guess straight into the double-float step
        no_fp32 = summary(timed(R.SWEEP_WARMSTART))
        ctx.set_warmstart(wts, R.DEFAULT_POLISH)  # network + FP32 steps, no double-float step
        no_dd = summary(timed(R.SWEEP_WARMSTART))
        ctx.set_warmstart(None, R.DEFAULT_START)
        base = {"value": value, "ms_per_step": ms_step, "mean_newton_iters": main_r["mean_iters"],
                "mean_fp32_steps": main_r["mean_f32"]}
        warm.update({
            "what": "network guess per (node, phase) on the tensor cores (per-warp mma.sync m16n8k16 BF16, FP32 "
                    "accumulation) inside the sweep, then up to 4 FP32 Newton steps and the double-float Halley "
                    "step; the FP64 Newton runs to the reference's tolerance from there",
            "pairs": 8_000_000, "collect_s": t1 - t0, "train_s": train_s, "final_train_loss": float(loss[-1]),
            "speedup_vs_reference_start": warm["value"] / ref_r["value"],
            "iteration_ratio_vs_reference_start": ref_r["mean_newton_iters"] / warm["mean_newton_iters"],
            "speedup_vs_default_start": warm["value"] / value,
            "ablation": {
                "default_start_no_network": base,
                "network_tcgen05_tiles": tiles_s,
                "network_then_double_float_only": no_fp32,
                "network_then_fp32_only": no_dd,
                "fp32_steps_only_no_network": fp32_r}})

    # ---- RheologicalOperators, Newton form: 8 perturbed local solves per node and phase ----
    newton_op = None
    if not args.no_operators:
        ops = R.alloc_operator_fields(w.Nc, w.Nv, like=d["eta_n"])
        sweep(w.model, w.mat, fs, mem=R.MEM_DEVICE)  # the state the operator linearises
        for _ in range(args.warmup):
            ctx.operators(w.model, w.mat, fs, ops, jacobian=1, aniso=aniso, mem=R.MEM_DEVICE)
        barrier()
        op_ms, op_calls = [], 0
        e0.record(stream)
        for _ in range(args.steps):
            _, ost = ctx.operators(w.model, w.mat, fs, ops, jacobian=1, aniso=aniso, mem=R.MEM_DEVICE)
            op_ms.append(ost.elapsed_ms)
            op_calls = ost.phase_calls
        e1.record(stream)
        barrier()
        ms_op = REP.max_over_ranks(e0.elapsed_time(e1), dev) / args.steps
        newton_op = {"what": "RheologicalOperators(Jacobian=1): D tensors with finite-difference derivatives, "
                             "8 perturbed local solves per node and active phase"
                             + ("" if aniso else "; plastic returns compacted per CTA"),
                     "ms_per_launch": ms_op, "node_updates_per_s": REP.whole_job_rate(w.nodes, ws, ms_op),
                     "local_solves_per_launch": int(op_calls),
                     "local_solves_per_s": op_calls * ws / (ms_op * 1e-3)}
        if not aniso:  # the same operator one thread per node, for comparison
            ctx.operators(w.model, w.mat, fs, ops, jacobian=1, mem=R.MEM_DEVICE, flags=R.OPS_PER_NODE)
            barrier()
            e0.record(stream)
            for _ in range(args.steps):
                ctx.operators(w.model, w.mat, fs, ops, jacobian=1, mem=R.MEM_DEVICE, flags=R.OPS_PER_NODE)
            e1.record(stream)
            barrier()
            newton_op["one_thread_per_node_ms_per_launch"] = REP.max_over_ranks(e0.elapsed_time(e1), dev) / args.steps
        del ops

    # ---- StrainRateComponents on the same grid: the step before the sweep ----
    strain = None
    if not args.no_strain_rates:
        vf = W.velocity_field(seed=REP.replica_seed(9, rank), ncx=args.size)
        sr = {k: torch.from_numpy(v).to(dev) for k, v in vf.arrays.items()}
        sr_args = (vf.model, vf.info["dx"], vf.info["dz"], sr)
        for _ in range(max(3, args.warmup)):
            ctx.strain_rates(*sr_args, mem=R.MEM_DEVICE)
        barrier()
        reps = 20 * args.steps  # ~0.2 ms each: more launches for a stable mean
        sr_ms = []
        e0.record(stream)
        for _ in range(reps):
            _, sst = ctx.strain_rates(*sr_args, mem=R.MEM_DEVICE)
            sr_ms.append(sst.elapsed_ms)
        e1.record(stream)
        barrier()
        ms_sr = REP.max_over_ranks(e0.elapsed_time(e1), dev) / reps
        sr_launch_ms = statistics.mean(sr_ms)
        sr_bytes = strain_rate_bytes(vf.model.Nx, vf.model.Nz)
        strain = {"what": "StrainRateComponents: velocity gradients, divergence, deviatoric normal rates, shear "
                          "rate and spin, centroid averages and vertex interpolation in one launch",
                  "grid": f"{args.size}x{args.size} cells", "ms_per_call": ms_sr,
                  "kernel_ms_per_launch": sr_launch_ms,
                  "algorithmic_bytes_per_launch": sr_bytes,
                  "hbm_achieved_gbs": sr_bytes / (sr_launch_ms * 1e-3) / 1e9,
                  "l2": f"{sr_bytes / 1e9:.2f} GB per launch, larger than L2; no flush"}
        del sr, vf

    # ---- the sweep's input preparation on the same grid: Softening, ShearModCompExpGrid ----
    prep = None
    if not args.no_prep:
        pw = W.prep_workload(seed=REP.replica_seed(13, rank), ncx=args.size, nphases=args.phases)
        pd = {k: ([torch.from_numpy(x).to(dev) for x in v] if isinstance(v, list) else torch.from_numpy(v).to(dev))
              for k, v in pw.arrays.items()}
        pfs = R.PrepFieldSet(pd)
        steps = {"softening": lambda: ctx.softening(pw.model, pw.mat, pfs, marker_noise=1, mem=R.MEM_DEVICE),
                 "shear_modulus": lambda: ctx.shear_modulus(pw.model, pw.mat, pfs, mem=R.MEM_DEVICE)}
        prep = {}
        for name, call in steps.items():
            for _ in range(max(3, args.warmup)):
                call()
            barrier()
            reps = 20 * args.steps
            k_ms = []
            e0.record(stream)
            for _ in range(reps):
                _, pst = call()
                k_ms.append(pst.elapsed_ms)
            e1.record(stream)
            barrier()
            ms = REP.max_over_ranks(e0.elapsed_time(e1), dev) / reps
            nbytes = prep_bytes(name, pw.Nc, pw.Nv, args.phases)
            prep[name] = {"ms_per_call": ms, "kernel_ms_per_launch": statistics.mean(k_ms),
                          "algorithmic_bytes_per_launch": nbytes,
                          "hbm_achieved_gbs": nbytes / (statistics.mean(k_ms) * 1e-3) / 1e9}
        prep["grid"] = f"{args.size}x{args.size} cells, {args.phases} phases, piecewise-linear softening with marker noise"
        del pd, pfs, pw

    # ---- UpdateParticleStress: grid stress increments to the markers ----
    markers = None
    if not args.no_markers:
        mw = W.marker_workload(seed=REP.replica_seed(17, rank), ncx=args.size, markers_per_cell=16)
        gd = {k: torch.from_numpy(v).to(dev) for k, v in mw.arrays.items()}
        md = {k: torch.from_numpy(v).to(dev) for k, v in mw.info["markers"].items()}
        nmk = int(mw.info["markers"]["x"].size)
        markers = {"grid": f"{args.size}x{args.size} cells, 16 markers per cell ({nmk} markers, cell by cell), "
                           "2 % inactive, no air"}
        # (elastic, rotation, anisotropy, advection, stencil, subgrid_diffusion)
        variants = {"jaumann_stencil1": (1, 1, 0, 1, 1, 0), "analytical_director_stencil9": (1, 2, 1, 1, 9, 0),
                    "subgrid2_jaumann_stencil1": (1, 1, 0, 1, 1, 2)}
        for name, o in variants.items():
            opts = R.MarkerOpts()
            (opts.elastic, opts.stress_rotation, opts.anisotropy, opts.advection, opts.interp_stencil,
             opts.subgrid_diffusion) = o
            opts.set_G(mw.info["G"])
            call = lambda: ctx.marker_stress(mw.model, opts, gd, md, mw.info["dx"], mw.info["dz"], mem=R.MEM_DEVICE)
            for _ in range(max(3, args.warmup)):
                call()
            barrier()
            reps = 5 * args.steps
            k_ms = []
            e0.record(stream)
            for _ in range(reps):
                _, mst = call()
                k_ms.append(mst.elapsed_ms)
            e1.record(stream)
            barrier()
            ms = REP.max_over_ranks(e0.elapsed_time(e1), dev) / reps
            nbytes = marker_bytes(nmk, mw.model.Nx, mw.model.Nz, o[2] == 1)
            markers[name] = {"ms_per_call": ms, "kernel_ms_per_call": statistics.mean(k_ms), "markers_per_call": nmk,
                             "markers_per_s": REP.whole_job_rate(nmk, ws, ms),
                             "algorithmic_bytes_per_call": nbytes,
                             "hbm_achieved_gbs": nbytes / (statistics.mean(k_ms) * 1e-3) / 1e9}
        # the default options end to end on ordinary pageable host arrays, as the drop-in
        # passes them: read and written in place where the GPU reads pageable memory through
        # the host page tables, and staged through device copies (MDZ_SWEEP_STAGED)
        opts = R.MarkerOpts()
        (opts.elastic, opts.stress_rotation, opts.anisotropy, opts.advection, opts.interp_stencil,
         opts.subgrid_diffusion) = variants["jaumann_stencil1"]
        opts.set_G(mw.info["G"])
        gh = {k: v.copy() for k, v in mw.arrays.items()}
        mh = {k: v.copy() for k, v in mw.info["markers"].items()}
        for label, fl in (("e2e_pageable", 0), ("e2e_pageable_staged", R.SWEEP_STAGED)):
            ctx.marker_stress(mw.model, opts, gh, mh, mw.info["dx"], mw.info["dz"], flags=fl)
            barrier()
            reps = max(2, args.steps // 2)
            e0.record(stream)
            for _ in range(reps):
                _, hst = ctx.marker_stress(mw.model, opts, gh, mh, mw.info["dx"], mw.info["dz"], flags=fl)
            e1.record(stream)
            barrier()
            ms = REP.max_over_ranks(e0.elapsed_time(e1), dev) / reps
            markers["jaumann_stencil1"][label] = {
                "ms_per_call": ms, "markers_per_s": REP.whole_job_rate(nmk, ws, ms),
                "in_place": bool(fl == 0 and ctx.pageable_in_place()),
                "h2d_bytes_per_call": int(hst.h2d_bytes), "d2h_bytes_per_call": int(hst.d2h_bytes)}
        del gh, mh
        # P2Mastah of a marker array onto the centroids and the vertices (the plastic strain
        # of CohesionFrictionDilationGrid), device-resident
        vals = torch.rand(nmk, dtype=torch.float64, device=dev)
        node_n = torch.zeros((mw.model.Nx - 1) * (mw.model.Nz - 1), dtype=torch.float64, device=dev)
        node_s = torch.zeros(mw.model.Nx * mw.model.Nz, dtype=torch.float64, device=dev)
        for name, stencil in (("p2mastah_stencil1", 1), ("p2mastah_stencil9", 9)):
            call = lambda: ctx.p2mastah(mw.model, gd, md, vals, 0, stencil, node_n, node_s, mw.info["dx"],
                                        mw.info["dz"], mem=R.MEM_DEVICE)
            for _ in range(max(3, args.warmup)):
                call()
            barrier()
            reps = 5 * args.steps
            k_ms = []
            e0.record(stream)
            for _ in range(reps):
                _, pst = call()
                k_ms.append(pst.elapsed_ms)
            e1.record(stream)
            barrier()
            ms = REP.max_over_ranks(e0.elapsed_time(e1), dev) / reps
            markers[name] = {"what": "P2Mastah of one marker array onto the centroids and the vertices",
                             "ms_per_call": ms, "kernel_ms_per_call": statistics.mean(k_ms),
                             "markers_per_s": REP.whole_job_rate(nmk, ws, ms)}
        del gd, md, mw, vals, node_n, node_s

    # ---- the anisotropic sweep at 4097^2 and 64 uneven grids in one launch ----
    configs, mg_sample = None, None
    if not args.no_configs and not aniso:
        configs = {"aniso_4097": aniso_section(args, ctx, dev, ws, rank, stream, barrier, args.no_warm)}
        configs["many_grids_64"], mg_sample = many_grids_section(args, ctx, dev, ws, rank, stream, barrier,
                                                                 warm=not args.no_warm)

    if rank != 0:
        REP.finalize()
        return

    # ---- roofline of the dominant kernel (k_sweep) ----
    launch_ms = statistics.mean(kernel_ms)
    peak_fp64 = R.measure_fp64_peak(dev)
    default_phases = {"plain_large": 5, "aniso": 3}
    if args.workload in FP64_FLOPS_PER_POINT and args.phases == default_phases[args.workload]:
        achieved = FP64_FLOPS_PER_POINT[args.workload] * w.nodes / (launch_ms * 1e-3) / 1e12
        roof = {"bound": "fp64", "achieved": achieved, "peak": peak_fp64, "unit": "TFLOP/s",
                "frac": achieved / peak_fp64, "peak_source": "measured (DFMA probe, mdz_rheo_measure_fp64_peak)",
                "traffic": (DRAM_BYTES_PER_POINT[args.workload] * w.nodes
                            if DRAM_BYTES_PER_POINT[args.workload] else None),
                "fp64_issue_frac": issue_frac(FP64_THREAD_INSTS[args.workload], w.nodes, launch_ms, peak_fp64)}
    else:
        roof = {"bound": "fp64", "achieved": None, "peak": peak_fp64, "unit": "TFLOP/s", "frac": None,
                "peak_source": "measured (DFMA probe)", "traffic": None}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
        hbm = peaks.get("hbm_gbs")
    except Exception:
        hbm = None
    bytes_alg = algorithmic_bytes(w, aniso)
    roof["hbm_achieved_gbs"] = bytes_alg / (launch_ms * 1e-3) / 1e9
    roof["hbm_frac"] = (roof["hbm_achieved_gbs"] / hbm) if hbm else None
    roof["algorithmic_bytes_per_launch"] = bytes_alg
    if strain is not None:
        strain["hbm_frac"] = strain["hbm_achieved_gbs"] / hbm if hbm else None
    for v in list((prep or {}).values()) + list((markers or {}).values()):
        if isinstance(v, dict) and "hbm_achieved_gbs" in v:
            v["hbm_frac"] = v["hbm_achieved_gbs"] / hbm if hbm else None
    if newton_op is not None and not aniso:  # per perturbed local solve, isotropic operator
        solves, ms_op = newton_op["local_solves_per_launch"], newton_op["ms_per_launch"]
        fl_op = FP64_FLOPS_PER_OPERATOR_SOLVE * solves / (ms_op * 1e-3) / 1e12
        newton_op["roofline"] = {"bound": "fp64", "achieved": fl_op, "peak": peak_fp64, "unit": "TFLOP/s",
                                 "frac": fl_op / peak_fp64, "peak_source": "measured (DFMA probe)",
                                 "fp64_flops_per_solve": FP64_FLOPS_PER_OPERATOR_SOLVE,
                                 "fp64_issue_frac": issue_frac(FP64_THREAD_INSTS["newton_operator"], solves, ms_op,
                                                               peak_fp64)}
    for name, v in (markers or {}).items():
        if name in FP64_FLOPS_PER_MARKER:
            nmk = v["markers_per_call"]
            v["fp64_flops_per_marker"] = FP64_FLOPS_PER_MARKER[name]
            v["fp64_achieved_tflops"] = FP64_FLOPS_PER_MARKER[name] * nmk / (v["kernel_ms_per_call"] * 1e-3) / 1e12
            v["fp64_frac"] = v["fp64_achieved_tflops"] / peak_fp64
            v["fp64_issue_frac"] = issue_frac(FP64_THREAD_INSTS.get(name), nmk, v["kernel_ms_per_call"], peak_fp64)

    if configs is not None:
        a = configs["aniso_4097"]
        fl = FP64_FLOPS_PER_POINT["aniso"] * a["nodes"] / (a["kernel_ms_per_sweep"] * 1e-3) / 1e12
        a["roofline"] = {"bound": "fp64", "achieved": fl, "peak": peak_fp64, "unit": "TFLOP/s",
                         "frac": fl / peak_fp64, "peak_source": "measured (DFMA probe)",
                         "traffic": DRAM_BYTES_PER_POINT["aniso"] * a["nodes"],
                         "hbm_achieved_gbs": a["algorithmic_bytes_per_sweep"] / (a["kernel_ms_per_sweep"] * 1e-3) / 1e9,
                         "fp64_issue_frac": issue_frac(FP64_THREAD_INSTS["aniso"], a["nodes"],
                                                       a["kernel_ms_per_sweep"], peak_fp64)}
        m = configs["many_grids_64"]
        per_call = FP64_FLOPS_PER_PHASE_CALL["many_grids"]
        g = m["graph"]["default"]
        if per_call:
            fl = per_call * g["phase_calls_per_sweep"] / (g["ms_per_sweep"] * 1e-3) / 1e12
            m["roofline"] = {"bound": "fp64", "achieved": fl, "peak": peak_fp64, "unit": "TFLOP/s",
                             "frac": fl / peak_fp64, "peak_source": "measured (DFMA probe)", "traffic": None,
                             "fp64_issue_frac": issue_frac(FP64_THREAD_INSTS["many_grids"],
                                                           g["phase_calls_per_sweep"], g["ms_per_sweep"], peak_fp64)}
        else:
            m["roofline"] = {"bound": "fp64", "achieved": None, "peak": peak_fp64, "unit": "TFLOP/s", "frac": None,
                             "peak_source": "measured (DFMA probe)", "traffic": None}
    cpu = None
    if not args.no_cpu_baseline and ws == 1:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        try:
            import oracle_lib as O
            O.build(ref=False)
            cpu = cpu_baseline(W, O, aniso=aniso)
            if markers is not None:
                markers["cpu_baseline"] = marker_cpu_baseline(W, O)
            if configs is not None:
                configs["aniso_4097"]["cpu_baseline"] = cpu_baseline(W, O, aniso=True)
                configs["many_grids_64"]["cpu_baseline"] = many_grids_cpu_baseline(O, mg_sample)
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": UNIT, "cores": None, "kind": "port", "sample": f"failed: {e}"}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": (f"aniso: {args.size}x{args.size} cells, {args.phases} phases (dislocation, "
                                    "softened Drucker-Prager), director angle U[0,pi), anisotropy factor "
                                    "log-U(1,10)" if aniso else
                                    f"plain_large: {args.size}x{args.size} cells, {args.phases} phases "
                                    "(dislocation, diffusion, Peierls, softened Drucker-Prager)")
                                   + "; FP64 local Newton to |r| < 1e-13 Eii started after up to 4 FP32 Newton "
                                     "steps and one double-float Halley step",
                       "nodes_per_gpu": w.nodes, "phase_calls_per_step": calls // args.steps,
                       "mean_newton_iters": main_r["mean_iters"], "max_newton_iters": main_r["maxit"],
                       "mean_fp32_steps": main_r["mean_f32"],
                       "l2": f"inputs larger than L2 ({algorithmic_bytes(w, aniso) / 1e9:.1f} GB moved per sweep), "
                             "no flush",
                       "parallelism": f"{ws} independent grid(s), one per GPU"},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk_summary,
            "gpu_launches": launches, "kernel_ms_per_sweep": launch_ms,
            "sweep_kernels": ("k_sweep over the centroids, then k_sweep over the vertices: 2 launches per sweep"
                              if aniso else
                              "k_sweep_compact over the centroids, then k_sweep_compact over the vertices "
                              "(plastic returns compacted per CTA): 2 launches per sweep"),
            "median_kernel_ms_per_sweep": statistics.median(kernel_ms),
            "reference_start": ref_r, "warm_start": warm, "autotune": tune, "newton_operator": newton_op,
            "strain_rates": strain, "input_preparation": prep, "marker_stress": markers, "configs": configs}
    print(json.dumps(line))
    if ws > 1:
        REP.finalize()


if __name__ == "__main__":
    main()
