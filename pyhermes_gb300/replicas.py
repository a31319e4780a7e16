"""Replica parallelism over several GPUs (one process per GPU).

The field pipeline has independent units (catalogues, samples) and no
exchange step, so N GPUs run N replicas: rank r takes every world-th unit,
nothing crosses ranks on the data path, and only the timing is combined
(the slowest rank's time; units summed) for a whole-job throughput.
"""

import torch


def shard(items, rank, world):
    """Rank `rank`'s share of a list of independent units (round robin)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of world {world}")
    return list(items)[rank::world]


def _reduce(value, op, device=None):
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(value, device=None):
    """The largest value over all ranks (the whole job's wall time)."""
    import torch.distributed as dist

    return _reduce(value, dist.ReduceOp.MAX if dist.is_available() else None, device)


def sum_over_ranks(value, device=None):
    import torch.distributed as dist

    return _reduce(value, dist.ReduceOp.SUM if dist.is_available() else None, device)


def job_throughput(units_local, seconds_local, device=None):
    """(units over all ranks, slowest rank's seconds, units per second)."""
    units = sum_over_ranks(units_local, device)
    seconds = max_over_ranks(seconds_local, device)
    return units, seconds, units / seconds if seconds > 0 else float("inf")
