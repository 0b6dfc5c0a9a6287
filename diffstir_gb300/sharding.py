"""Scene sharding across GPUs (one process per GPU).

Scenes (or identification candidates) are independent: a rank simulates a
contiguous range of them and nothing crosses ranks in the data path.  The only
exchange is after a gradient evaluation, when every rank needs the
[B, 4] parameter gradients and [B] losses of all scenes (an all-gather of a few
hundred bytes), e.g. to pick the best restart.
"""

import numpy as np


def shard_range(n_items, world, rank):
    """Contiguous, balanced [start, stop) of ``n_items`` for ``rank`` of ``world``."""
    base, rem = divmod(int(n_items), int(world))
    start = rank * base + min(rank, rem)
    stop = start + base + (1 if rank < rem else 0)
    return start, stop


def allgather_rows(local, n_items, group=None):
    """All-gather per-rank row blocks (shard_range layout) into [n_items, ...].

    ``local`` is a torch tensor holding this rank's rows; uses
    torch.distributed (any backend; gloo on CPU, NCCL on GPU)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    counts = [shard_range(n_items, world, r) for r in range(world)]
    width = max(b - a for a, b in counts)
    pad = torch.zeros((width,) + tuple(local.shape[1:]), dtype=local.dtype, device=local.device)
    a, b = counts[rank]
    pad[:b - a] = local
    bufs = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(bufs, pad, group=group)
    rows = [bufs[r][:counts[r][1] - counts[r][0]] for r in range(world)]
    return torch.cat(rows, 0)


def max_over_ranks(value, group=None):
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def shard_seeds(n_scenes, world, rank, seed0=0):
    a, b = shard_range(n_scenes, world, rank)
    return list(np.arange(a, b) + seed0)
