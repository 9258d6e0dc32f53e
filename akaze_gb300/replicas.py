"""Replica bookkeeping for multi-GPU runs (one process per GPU).

A-KAZE images are independent, so N GPUs run N replicas: rank r processes its
own share of the images and no tensor crosses ranks on the data path.  The
only collective is the timing reduction (max over ranks) used to report a
whole-job throughput.
"""


def shard(items, rank, world):
    """Contiguous, balanced share of `items` for `rank` of `world`."""
    n = len(items)
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return items[start:stop]


def rank_seeds(rank, count, stride=10000):
    """Seeds of the synthetic images of one rank (distinct across ranks)."""
    return [stride * rank + i for i in range(count)]


def max_over_ranks(value, dist=None, device=None):
    """Largest value over all ranks (the job takes as long as its slowest rank)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world, seconds_max):
    """Whole-job units per second: all ranks' units over the slowest rank's time."""
    return units_per_rank * world / seconds_max
