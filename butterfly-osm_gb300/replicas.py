"""Multi-GPU form of the path: independent replicas, no data-path collective.

Matrix rows (source batches) and isochrone origins are independent units, so
N GPUs run N replicas of the engine, one process per GPU. Each rank either
runs its own seeded workload (weak scaling, what bench.py reports) or takes a
contiguous shard of one request's sources (shard()); the only collectives
are the timing barrier and the max over ranks of the measured time.
"""


def shard(n_units, rank, world):
    """Contiguous [begin, end) slice of n_units for this rank; the first
    n_units % world ranks take one unit more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside world of %d" % (rank, world))
    base, extra = divmod(int(n_units), int(world))
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def max_over_ranks(x, dist=None, device="cpu"):
    """Max of a float over all ranks (identity without a process group)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, seconds_max):
    """Units processed by all ranks divided by the slowest rank's time."""
    return world * units_per_rank / seconds_max
