"""Independent replicas on several GPUs: the host side of a multi-GPU run.

The MFV step of one simulation runs on one GPU; there is no data exchange
between GPUs (the reference is serial and its configurations fit one GPU).
Several GPUs run independent replicas (one process per GPU, launched by
torchrun): different seeds of the same workload, or disjoint shares of an
ensemble's members.  The only collectives are the timing barrier and the
max-over-ranks of the timed region, on the gloo backend (host values).
"""
from __future__ import annotations

import os


def dist_env():
    """(world size, rank, local rank) from the torchrun environment (1, 0, 0 alone)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(base: int, rank: int) -> int:
    """Seed of a rank's replica: every rank runs its own initial conditions."""
    return base + rank


def job_seconds(local_seconds: float, dist=None) -> float:
    """The whole job's time: the slowest rank's (max over ranks)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(local_seconds)
    import torch
    t = torch.tensor([float(local_seconds)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, seconds: float) -> float:
    """Whole-job throughput: the units all ranks processed over the job's time."""
    return float(sum(units_per_rank)) / seconds


def gather_units(local_units: float, dist=None):
    """Units processed by every rank (a list of world-size numbers)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return [float(local_units)]
    import torch
    ws = dist.get_world_size()
    t = torch.zeros(ws, dtype=torch.float64)
    t[dist.get_rank()] = float(local_units)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return [float(v) for v in t.tolist()]

