"""Scene sharding across GPUs (one process per GPU).

Scenes (or identification candidates) are independent: a rank simulates a
contiguous range of them and nothing crosses ranks in the data path.  The only
exchange is after a gradient evaluation, when every rank needs the
[B, 4] parameter gradients and [B] losses of all scenes (an all-gather of a few
hundred bytes), e.g. to pick the best restart.  The identification driver
(identify.adam_identify / clip_identify) shards its restarts this way when
torch.distributed is initialised.
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
    dev = comm_device(group)
    pad = torch.zeros((width,) + tuple(local.shape[1:]), dtype=local.dtype, device=dev)
    a, b = counts[rank]
    pad[:b - a] = local.to(dev)
    bufs = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(bufs, pad, group=group)
    rows = [bufs[r][:counts[r][1] - counts[r][0]] for r in range(world)]
    return torch.cat(rows, 0).to(local.device)


def active(group=None):
    """(world, rank) of ``group`` when torch.distributed is initialised,
    else (1, 0)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        return dist.get_world_size(group), dist.get_rank(group)
    return 1, 0


def comm_device(group=None):
    """Device of the tensors handed to the collectives: the current CUDA
    device under NCCL, the CPU otherwise (gloo)."""
    import torch
    import torch.distributed as dist
    if dist.get_backend(group) == 'nccl':
        return torch.device('cuda', torch.cuda.current_device())
    return torch.device('cpu')


def max_over_ranks(value, group=None):
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], device=comm_device(group))
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def sum_over_ranks(value, group=None):
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=comm_device(group))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return float(t.item())


def broadcast_tensor(t, src=0, group=None):
    """``t`` of rank ``src`` on every rank (same shape and dtype on all
    ranks); returned on ``t``'s device."""
    import torch.distributed as dist
    buf = t.detach().to(comm_device(group)).contiguous()
    dist.broadcast(buf, src=src, group=group)
    return buf.to(t.device)


def shard_seeds(n_scenes, world, rank, seed0=0):
    a, b = shard_range(n_scenes, world, rank)
    return list(np.arange(a, b) + seed0)
