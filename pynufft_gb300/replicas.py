"""Replica parallelism across GPUs: one process per GPU, independent units.

NUFFT work shards by independent units (coils, instances, whole transforms):
no unit needs data from another GPU, so there is no collective on the data
path.  The only cross-rank traffic is host-side bookkeeping: the slowest
rank's elapsed time and the total of units processed, so throughput is
reported for the whole job.
"""
from __future__ import annotations


def shard(n_units: int, rank: int, world: int):
    """Contiguous [start, stop) share of n_units for `rank` of `world`
    (the first n_units % world ranks take one extra unit)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError('need 0 <= rank < world')
    base, extra = divmod(int(n_units), world)
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return start, stop


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank float over the default process group (identity
    without one).  Works with gloo (CPU tensors) and nccl (device tensors)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def job_rate(units_this_rank: float, seconds_this_rank: float, device=None) -> float:
    """Whole-job throughput: total units over all ranks / slowest rank's time."""
    total = sum_over_ranks(units_this_rank, device)
    t = max_over_ranks(seconds_this_rank, device)
    return total / t if t > 0 else float('inf')
