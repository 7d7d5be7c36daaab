"""Several GPUs as independent replicas.

The solver step has no data-parallel split that keeps it exact (a sweep
reads its neighbours every iteration), so N GPUs run N independent
simulations: rank r advances its own grid with its own seeded obstacles and
forcing, and no collective touches the data path.  The only cross-rank
traffic is timing: the job's time is the slowest rank's, and the job's rate
is the units all ranks processed over that time (weak scaling).
"""
from __future__ import annotations


def replica_seed(rank: int) -> int:
    """Seed of rank `rank`'s synthetic workload (obstacles and forcing)."""
    return int(rank)


def max_over_ranks(values, device=None) -> list:
    """Element-wise maximum of `values` over the ranks of the default process
    group (the values themselves when there is no group or one rank)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def whole_job_rate(units_per_rank: float, world: int, slowest_seconds: float) -> float:
    """Units processed by all `world` ranks over the slowest rank's time."""
    return float(units_per_rank) * int(world) / float(slowest_seconds)
