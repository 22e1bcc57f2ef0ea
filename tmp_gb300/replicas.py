"""Whole-job rate of a multi-GPU run.

One GB300 holds every configuration of this solver, so a run on N GPUs is N
independent replicas (one process per GPU, each stepping its own copy of the
workload; no collective on the data path).  The only collective is the timing
reduction: the job's time is the slowest rank's, and its rate counts the work
of all ranks.
"""
from __future__ import annotations


def job_rate(units_per_rank: float, seconds_local: float, world: int, dist=None, device="cpu"):
    """(t_max, units per second of the whole job): t_max = max over ranks of
    seconds_local (all_reduce MAX when dist is an initialised torch.distributed
    and world > 1), rate = units_per_rank * world / t_max."""
    import torch

    t = torch.tensor([float(seconds_local)], dtype=torch.float64, device=device)
    if dist is not None and world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    t_max = float(t.item())
    return t_max, units_per_rank * world / t_max
