"""Multi-GPU layout of the path: cosmologies sharded over ranks.

Modes (cosmology x k) are independent, so each rank integrates its own
slice of the cosmology sample and no collective touches the data path; only
the step time is reduced (max over ranks) for reporting.  One process per
GPU, rank/world from the torchrun environment.
"""
from __future__ import annotations

import os


def dist_env():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(n_per_rank: int, world: int, rank: int) -> range:
    """Indices of the global cosmology sample owned by ``rank`` (weak scaling:
    every rank owns ``n_per_rank`` cosmologies)."""
    if not (0 <= rank < world) or n_per_rank < 0:
        raise ValueError("bad rank/world")
    return range(rank * n_per_rank, (rank + 1) * n_per_rank)


def max_over_ranks(value: float, device=None) -> float:
    """Largest value over all ranks (the job's step time)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
