"""Whole-job timing across replica ranks (one independent target per GPU).

The block-DDA solve path does not shard a single target; N GPUs run N
independent solves.  The job's time is the slowest rank's, and its throughput
is the work of all ranks over that time.  Works with any initialised
torch.distributed backend (NCCL on GPUs, gloo in the CPU tests) and degrades to
the local value when no process group is initialised.
"""
from __future__ import annotations


def max_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, max_time_s: float, world_size: int) -> float:
    """Units processed by all ranks per second of the slowest rank."""
    return units_per_rank * world_size / max_time_s
