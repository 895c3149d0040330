"""Sharding a render or a job list over replicas (one process per GPU).

Path samples and jobs are independent, so replicas exchange nothing while
they render.  One image split by sample range needs a single exchange at
the end: the films (rgb sum, weight per pixel) add up, because every
sample's contribution lands in the same pixel whichever replica rendered it
(Screen::merge adds per-tile screens the same way, core/Screen.cpp:136-157).
A job list is split by job, with no exchange at all.
"""


def sample_range(spp, rank, world):
    """Contiguous share of samples [begin, begin + count) for `rank`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(int(spp), world)
    begin = rank * base + min(rank, extra)
    return begin, base + (1 if rank < extra else 0)


def partition_jobs(costs, world):
    """Assign jobs to ranks, largest first onto the least-loaded rank.
    Returns one list of job indices per rank (deterministic)."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += costs[i]
    return out


def reduce_films(film, group=None):
    """Sum a film tensor over all ranks in place (the one exchange step)."""
    import torch.distributed as dist
    dist.all_reduce(film, op=dist.ReduceOp.SUM, group=group)
    return film
