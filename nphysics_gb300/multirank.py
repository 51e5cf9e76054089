"""Several GPUs of one node, one process each (launched by torchrun).

Batched worlds shard with no data-path exchange: each rank takes a
contiguous range of the batch's worlds and steps them on its own GPU. A
single large world does not shard; ranks then run replicas. The only
collectives are on the host side of the measurement: a barrier around the
timed region and the maximum of the ranks' times.
"""
import os


def rank_env():
    """(rank, world_size, local_rank) from the torchrun environment (1 process
    without it)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(n_items, rank, world_size):
    """The contiguous range of n_items that rank owns; ranges are disjoint,
    cover every item, and differ in length by at most one."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("rank outside the world")
    base, extra = divmod(n_items, world_size)
    lo = rank * base + min(rank, extra)
    return range(lo, lo + base + (1 if rank < extra else 0))


def reduce_max(value, device=None):
    """The largest value over all ranks (value itself with one process)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(value, device=None):
    """The sum of value over all ranks."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(units_per_rank, seconds_per_rank, device=None):
    """Units all ranks processed over the slowest rank's time: the whole-job
    throughput a multi-GPU run reports."""
    total = reduce_sum(units_per_rank, device)
    slowest = reduce_max(seconds_per_rank, device)
    return total / slowest if slowest > 0 else 0.0
