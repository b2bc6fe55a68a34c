"""Point shards for one process per GPU.

Points are independent, so N GPUs each take a contiguous range of the point
index space and nothing is exchanged on the data path.  ``rank_points`` gives
the weak-scaling layout (every rank owns ``per_rank`` points, rank r starting
at r * per_rank); ``split_points`` the strong-scaling one (a fixed total split
as evenly as possible).  ``max_over_ranks`` is the only collective: the
timing reduction of the benchmark.
"""


def rank_points(per_rank, rank):
    """(first, count) of rank `rank` when every rank owns `per_rank` points."""
    if per_rank < 0 or rank < 0:
        raise ValueError("per_rank and rank must be >= 0")
    return rank * per_rank, per_rank


def split_points(total, rank, world):
    """(first, count) of rank `rank` of `world` for `total` points in all."""
    if world < 1 or not 0 <= rank < world or total < 0:
        raise ValueError("need 0 <= rank < world and total >= 0")
    base, extra = divmod(total, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def max_over_ranks(value, device=None):
    """Maximum of a float over the ranks of the default process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
