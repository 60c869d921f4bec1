"""Independent-replica execution across ranks (no data-path collective).

A batch of reconstructions shards across ranks by case; nothing is exchanged
between ranks except the timing and counts used for reporting (a host-side
max / sum at the end).  One reconstruction never spans ranks.
"""
from __future__ import annotations

import os
from typing import List, Sequence, Tuple


def env() -> Tuple[int, int, int]:
    """(world_size, rank, local_rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(items: Sequence, rank: int, world: int) -> List:
    """Round-robin share of `items` for `rank` (every item exactly once overall)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return [it for k, it in enumerate(items) if k % world == rank]


def case_seed(base_seed: int, rank: int, case: int = 0) -> int:
    """Distinct, reproducible phantom seed per (rank, case)."""
    return int(base_seed) + 1000 * int(rank) + int(case)


def reduce_timing(elapsed_s: float, units: float, group=None) -> Tuple[float, float]:
    """(max elapsed over ranks, total units over ranks).  Single process: identity."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(elapsed_s), float(units)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(elapsed_s)], dtype=torch.float64, device=dev)
    u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
    return float(t.item()), float(u.item())
