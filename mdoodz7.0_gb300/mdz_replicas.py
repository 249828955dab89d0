"""Replica runs over several GPUs: one independent grid per rank.

The local rheology update has no exchange step between grids (each node needs only
its own fields and, at vertices, its four ring centroids), so N GPUs run N
independent sweeps: no data-path collective, weak scaling.  The only collective is
the MAX over ranks of a timed region, so that a whole-job rate is the nodes of all
ranks over the slowest rank's time.  Works with `nccl` (CUDA tensors) and `gloo`
(CPU tensors).
"""
from __future__ import annotations

import os
from typing import Optional, Tuple


def dist_env() -> Tuple[int, int, int]:
    """(world_size, rank, local_rank) from the torchrun environment (1, 0, 0 without)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str = "nccl") -> None:
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend)


def finalize() -> None:
    import torch.distributed as dist
    if dist.is_initialized():
        dist.destroy_process_group()


def replica_seed(base: int, rank: int) -> int:
    """Each rank sweeps its own grid: seeds base, base + 1, ..."""
    return base + rank


def max_over_ranks(value: float, device: Optional[object] = None) -> float:
    """MAX of a per-rank float over all ranks (the value itself when not distributed)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(nodes_per_rank: int, world_size: int, slowest_ms: float) -> float:
    """Point-updates/s of the whole job: every rank's nodes over the slowest rank's time."""
    return world_size * nodes_per_rank / (slowest_ms * 1e-3)
