"""Scene sharding host logic with two gloo ranks on CPU: each rank computes the
oracle gradients of its shard of scenes, the all-gather reassembles exactly the
single-process result, and the max-over-ranks timing reduction works."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from diffstir_gb300 import sharding


def test_shard_range_covers_and_balances():
    for n in (0, 1, 5, 64, 67):
        for world in (1, 2, 3, 8):
            spans = [sharding.shard_range(n, world, r) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def _scene_grads(seed):
    import oracle
    from diffstir_gb300 import scene as S
    T = 5
    sc = S.small_synthetic_scene(n_grid=10, ppc=1, n_steps=T, seed=int(seed), dt=5e-4,
                                 params=(0.4 + 0.1 * int(seed), 0.0, 0.7, 0.0))
    w = np.random.default_rng(int(seed)).normal(size=(T, 3))
    _, dp, _, _ = oracle.grad(sc.desc, sc.params, sc.trajectory, T, sc.x0(), w)
    return dp


def _worker(rank, world, port, n_scenes, out):
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    a, b = sharding.shard_range(n_scenes, world, rank)
    local = torch.tensor(np.stack([_scene_grads(s) for s in range(a, b)]) if b > a else np.zeros((0, 4)))
    full = sharding.allgather_rows(local, n_scenes)
    t = sharding.max_over_ranks(1.0 + rank)
    if rank == 0:
        torch.save({'full': full, 'max': t}, out)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_rank_gloo_sharded_gradients(tmp_path):
    import oracle
    oracle.build()
    n_scenes = 5
    out = str(tmp_path / 'res.pt')
    mp.start_processes(_worker, args=(2, _free_port(), n_scenes, out), nprocs=2, start_method='spawn')
    res = torch.load(out)
    ref = np.stack([_scene_grads(s) for s in range(n_scenes)])
    np.testing.assert_allclose(res['full'].numpy(), ref, rtol=0, atol=0)
    assert res['max'] == 2.0
