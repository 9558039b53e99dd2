"""Replica helpers for N GPUs (one process per GPU).

The path shards with no data exchange: every rank checks its own batch
against its own copy of the robot and scenes.  The only collective is the
max-over-ranks of the timed region (the job is as slow as its slowest rank).
"""


def shard(n, rank, world):
    """Contiguous [begin, end) of n items for this rank."""
    per = (n + world - 1) // world
    b = min(n, rank * per)
    return b, min(n, b + per)


def max_over_ranks(value, device=None):
    """Maximum of a float over all ranks (identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
