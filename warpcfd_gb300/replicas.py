"""Replica (one case or one request stream per GPU) helpers.

A single case does not shard without domain decomposition, so runs on N GPUs are N
replicas: each rank solves its own case, or serves its own share of the requests, with no
data-path collective.  The only cross-rank step is the timing: the job's time is the
slowest rank's, and its throughput is every rank's units over that time.
"""
from __future__ import annotations

import torch


def max_over_ranks(value: float, device=None) -> float:
    """The largest ``value`` over the ranks of the default process group (``value`` itself
    when torch.distributed is not initialised)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    """The sum of ``value`` over the ranks of the default process group."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def shard(items, rank: int, world: int):
    """Round-robin share of ``items`` for ``rank`` of ``world`` (every item exactly once
    over the ranks, shares differing in size by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    return list(items)[rank::world]


def job_throughput(units_per_rank: float, world: int, slowest_seconds: float) -> float:
    """Whole-job throughput of ``world`` replicas that each processed ``units_per_rank``."""
    return world * units_per_rank / max(slowest_seconds, 1e-300)
