"""Replica (batch-sharded) execution across GPUs.

Every benchmark configuration is a batch of independent problems, so N GPUs
run N independent shards with no data-path collective: each rank takes its own
problems (distinct seeds or a contiguous slice of a global batch), times its
own work, and rank 0 reports the whole-job throughput from the slowest rank.
The only communication is one scalar MAX reduction of the elapsed time.
(jaxfun's multi-device path is a slab all-to-all per transform,
src/jaxfun/sharding.py:43-105; none of the batched workloads needs it.)
"""

from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass(frozen=True)
class RankInfo:
    rank: int
    world: int
    local: int


def rank_info() -> RankInfo:
    return RankInfo(int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
                    int(os.environ.get("LOCAL_RANK", "0")))


def shard(total: int, rank: int, world: int) -> range:
    """Contiguous slice of a global batch of ``total`` problems for ``rank``."""
    base, extra = divmod(total, world)
    lo = rank * base + min(rank, extra)
    return range(lo, lo + base + (1 if rank < extra else 0))


def seed_base(rank: int, stride: int = 1000) -> int:
    """First problem seed of a rank's own (weak-scaling) batch."""
    return stride * rank


def max_time(t: float, dist=None, device=None) -> float:
    """MAX of the per-rank elapsed times (identity on one rank)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return t
    import torch

    tt = torch.tensor([t], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def throughput(units_per_rank: int, world: int, t_max: float) -> float:
    """Whole-job units per second: all ranks' units over the slowest rank's time."""
    return world * units_per_rank / t_max
