"""Multi-process helpers: one process per GPU, sub-volumes sharded across
ranks, no collective on the data path (sub-volumes with wide enough halos
evolve independently).  Only timing and bookkeeping cross ranks."""
from __future__ import annotations

import os
from typing import List, Sequence

from .tiling import Tile, lpt_shards


def rank_info():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(tiles: Sequence[Tile], rank: int, world: int) -> List[int]:
    """Tile indices this rank evolves (longest-processing-time by voxels)."""
    return lpt_shards(tiles, world)[rank]


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of `value` over all ranks (identity without a process group)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
