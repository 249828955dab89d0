"""The N > 1 path on CPU: two `gloo` ranks, each sweeping its own grid, joined only by
the MAX of their timed regions (mdz_replicas, as bench.py uses it under torchrun).
The sweeps run on the oracle here, because this host has no GPU; the aggregation and
the per-rank seeding are the code under test."""
import json
import os
import socket
import sys
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    for sub in ("mdoodz7.0_gb300", "oracle"):
        sys.path.insert(0, os.path.join(REPO, sub))
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import mdz_replicas as REP
    import mdz_rheo as R
    import mdz_workloads as W
    import oracle_lib as O
    REP.init("gloo")
    ws, r, _ = REP.dist_env()
    w = W.plain_small(seed=REP.replica_seed(1, r), ncx=24 + 8 * r)
    nodes = w.nodes
    t0 = time.perf_counter()
    rc, st = O.orc_sweep(w.model, w.mat, R.FieldSet(w.arrays))
    ms = (time.perf_counter() - t0) * 1e3 + 5.0 * r   # rank 1 is made the slower one
    slowest = REP.max_over_ranks(ms)
    REP.finalize()
    json.dump({"rank": r, "ws": ws, "rc": rc, "ms": ms, "slowest": slowest, "nodes": nodes,
               "eta0": float(w.arrays["eta_n"][0]), "calls": int(st.phase_calls)},
              open(os.path.join(outdir, f"rank{r}.json"), "w"))


def test_two_gloo_ranks_weak_scaling(tmp_path):
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    import mdz_replicas as REP
    assert all(x["ws"] == 2 and x["rc"] == 0 for x in res)
    slowest = max(x["ms"] for x in res)
    assert all(abs(x["slowest"] - slowest) < 1e-9 for x in res)       # every rank sees the MAX
    assert res[0]["eta0"] != res[1]["eta0"]                             # independent grids
    assert res[0]["calls"] > 0 and res[1]["calls"] > 0
    nodes = res[0]["nodes"]
    assert REP.whole_job_rate(nodes, 2, slowest) == pytest.approx(2 * nodes / (slowest * 1e-3))


def test_single_process_is_its_own_max():
    sys.path.insert(0, os.path.join(REPO, "mdoodz7.0_gb300"))
    import mdz_replicas as REP
    assert REP.max_over_ranks(3.5) == 3.5
    assert REP.replica_seed(1, 0) == 1 and REP.replica_seed(1, 3) == 4
