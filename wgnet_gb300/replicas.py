"""Replica runs over several GPUs of one node (one process per GPU, launched by torchrun).

The physics path does not shard: every (model, shot) unit is independent and a rank simply runs
its own batch (its own seeds), so there is no collective on the data path. The only exchanges
are for timing: a barrier before and after the timed region and the maximum of the ranks'
elapsed times, from which the whole-job throughput is the units of all ranks over that maximum.
"""

from __future__ import annotations

import os


def env() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment (single process: 0, 1, 0)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str = "nccl"):
    """Join the process group when more than one rank runs; returns torch.distributed or None."""
    _, world, _ = env()
    if world <= 1:
        return None
    import torch.distributed as dist

    if not dist.is_initialized():
        dist.init_process_group(backend)
    return dist


def barrier(dist) -> None:
    if dist is not None:
        dist.barrier()


def max_over_ranks(value: float, dist, device=None) -> float:
    """The largest `value` over all ranks (the timed region ends when the slowest rank ends)."""
    if dist is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: int, steps: int, world: int, max_ms: float) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return world * units_per_rank * steps / (max_ms / 1000.0)


def rank_seed(base: int, rank: int) -> int:
    """Each rank draws its own models (weak scaling: per-rank work fixed as ranks are added)."""
    return base + rank
