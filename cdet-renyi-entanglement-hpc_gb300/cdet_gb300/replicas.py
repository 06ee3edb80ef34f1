"""One replica of the tables per GPU: the host logic of a run on N GPUs.

The configurations of a step are independent, so a run on N GPUs is N
replicas, each evaluating its own batch (weak scaling), with no collective
on the data path: only a barrier around the timed region and the maximum of
the ranks' times. Ranks come from the torchrun environment (RANK,
LOCAL_RANK, WORLD_SIZE); each rank draws its configurations from its own
seed stream.
"""
from __future__ import annotations

import os
from typing import Tuple

from .synthetic import derive_seed

BATCH_SEED = 20261203  # base seed of the benchmark's configuration batches


def rank_info() -> Tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def batch_seed(rank: int, step: int) -> int:
    """Seed of a rank's configuration batch for a step (distinct per rank and
    step, the same on every run)."""
    return derive_seed(BATCH_SEED, 100 + rank, step)


def max_over_ranks(x: float, world: int, device=None) -> float:
    """The maximum of x over the ranks of the default process group (x itself
    when world == 1). device: where the reduction tensor lives (a CUDA device
    for NCCL, None for gloo)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank_step: int, steps: int, world: int, seconds: float) -> float:
    """Whole-job rate: every rank's units over the slowest rank's time."""
    return units_per_rank_step * steps * world / seconds
