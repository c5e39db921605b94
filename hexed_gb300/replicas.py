"""Replica harness of the benchmark: one independent solve per GPU, no data-path collective.

A solve does not shard in this library, so N GPUs run N replicas of the workload (weak
scaling). The only collectives are the timing barrier and the maximum of the elapsed time
over ranks; the job's rate is the work of all ranks over that maximum.
"""
from __future__ import annotations


def max_over_ranks(value, device="cpu"):
    """Maximum of a float over all ranks of the default process group (the value itself
    when no group is initialised)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, elapsed_ms):
    """Whole-job rate in units per second: every rank processed units_per_rank in at most
    elapsed_ms (the maximum over ranks)."""
    return units_per_rank * world / (elapsed_ms / 1e3)
