"""Replicas over the GPUs of one node.

A window's levels run one after another and each level reads nets of any
earlier level, so one window does not split across GPUs without an exchange
per level; independent windows split with none.  Every rank therefore
simulates its own window (its own stimulus seed) on its own GPU, with no
collective on the data path.  Timing takes the maximum over the ranks, and
the whole-job rate counts the work of every rank (weak scaling).
"""
from __future__ import annotations

import os


def world_rank() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def rank_seed(seed: int, rank: int) -> int:
    """The stimulus seed of a rank's window (every rank a different window)."""
    return seed + 1 + 1000 * rank


def max_over_ranks(x: float, device: str = "cpu") -> float:
    """The largest x over the ranks of the default process group (x itself
    without one).  device: where the reduction tensor lives ("cuda" for
    NCCL, "cpu" for gloo)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units of all ranks (each did units_per_rank) over the slowest rank's time."""
    return units_per_rank * world / seconds


def partition_windows(work, world: int) -> list[list[int]]:
    """Independent stimulus windows split over `world` ranks by predicted
    work (e.g. the window's length in cycles): longest first, each to the
    rank with the least work so far (ties to the lower rank).  Every rank
    gets its windows in increasing index order; the split is the same on
    every rank, so no exchange is needed to agree on it."""
    import heapq
    order = sorted(range(len(work)), key=lambda k: (-float(work[k]), k))
    heap = [(0.0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for k in order:
        load, r = heapq.heappop(heap)
        out[r].append(k)
        heapq.heappush(heap, (load + float(work[k]), r))
    return [sorted(x) for x in out]
