"""Replica runs across ranks (one process per GPU).

A steady solve does not shard: its sweep couples every element of the mesh
through the upwind dependencies, and its outer iteration needs every
ordinate's moments.  Several GPUs therefore run independent replicas of
the workload, one process per GPU with no data-path collective; the only
collectives are the timing barrier and the max-over-ranks of the elapsed
time, so the throughput of N replicas is ``N * solves / max_rank_seconds``
(weak scaling: the work per GPU is fixed as N grows).
"""
from __future__ import annotations

import os

import torch

__all__ = ["RankInfo", "rank_info", "max_over_ranks", "replica_throughput", "barrier"]


class RankInfo:
    def __init__(self, world: int, rank: int, local: int):
        self.world, self.rank, self.local = world, rank, local

    @property
    def is_root(self) -> bool:
        return self.rank == 0


def rank_info(env=None) -> RankInfo:
    """WORLD_SIZE / RANK / LOCAL_RANK from the launcher (1 / 0 / 0 alone)."""
    env = os.environ if env is None else env
    return RankInfo(int(env.get("WORLD_SIZE", "1")), int(env.get("RANK", "0")), int(env.get("LOCAL_RANK", "0")))


def _tensor_device(dist):
    if dist is not None and dist.is_initialized() and dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def barrier(dist=None) -> None:
    """Process-group barrier (when there is one), then the local device."""
    if dist is not None and dist.is_initialized():
        dist.barrier()
    if torch.cuda.is_available() and torch.cuda.is_initialized():
        torch.cuda.synchronize()


def max_over_ranks(value: float, dist=None) -> float:
    """The largest ``value`` over all ranks (the value itself alone)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=_tensor_device(dist))
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: int, max_seconds: float, world: int) -> float:
    """Whole-job units per second of ``world`` replicas, each of which did
    ``units_per_rank`` units, the slowest in ``max_seconds``."""
    if max_seconds <= 0:
        raise ValueError("elapsed time must be positive")
    return world * units_per_rank / max_seconds
