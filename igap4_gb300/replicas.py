"""Replica bookkeeping for runs with one process per GPU.

The assembly path is not sharded here: every rank assembles its own copy of
the problem and the ranks exchange nothing but timings.  The slowest rank's
device time per step defines the whole-job rate (units of all ranks divided
by that time).
"""
from __future__ import annotations


def max_over_ranks(value: float, device=None) -> float:
    """Largest `value` over the ranks of the default process group (the value
    itself without one, or with one rank)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, ms_per_step: float, world: int) -> float:
    """Whole-job throughput: world x units per rank per step / slowest step time."""
    return world * units_per_rank / (ms_per_step * 1e-3)
