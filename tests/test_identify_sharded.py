"""Rank-sharded identification with two gloo ranks on CPU.

The identification driver of the reference runs its restarts and epochs in
one process (src/gradient_descent_module.py:99-139).  Here adam_identify
splits the restarts over the ranks of an initialised process group (each rank
one batched handle, nothing exchanged until the end) and all-gathers the best
parameters, losses and histories; clip_identify carries rank 0's roll-forward
state to every rank.  The simulator is the differentiable stand-in of
test_identify_host.py, so the sharded run must reproduce the single-process
run of the same restarts exactly."""

import os
import socket

import numpy as np
import torch
import torch.multiprocessing as mp

from diffstir_gb300 import identify
from diffstir_gb300 import scene as S

import test_identify_host as H


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _setup_fakes(clip=False):
    identify.Simulator = H.FakeClipSim if clip else H.FakeSim
    torch.cuda.synchronize = lambda *a, **k: None


def _adam_case():
    T = 30
    sc = S.small_synthetic_scene(n_grid=8, ppc=1, n_steps=T, seed=0)
    return sc, H._target((1.1, 0.0, 0.65, 0.0), T)


def _clip_case():
    T, fpc = 30, 10
    sc = S.small_synthetic_scene(n_grid=8, ppc=1, n_steps=T, seed=0)
    return sc, H._target((1.0, 0.0, 0.7, 0.0), T), fpc


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    _setup_fakes()
    sc, tgt = _adam_case()
    seen = []
    res = identify.adam_identify(sc, tgt, restarts=5, iters=40, lr=5e-2, free=(0, 2), seed=7,
                                 init_params=(0.5, 0.0, 1.0, 0.0), callback=lambda it, p, lv: seen.append(len(lv)))
    _setup_fakes(clip=True)
    sc2, tgt2, fpc = _clip_case()
    clips = identify.clip_identify(sc2, tgt2, fpc, carry='full', restarts=3, iters=3, lr=1e-2, free=(0, 2))
    torch.save({'best_params': res['best_params'], 'best_loss': res['best_loss'], 'history': res['history'],
                'best_index': res['best_index'], 'range': res['restart_range'], 'local': seen[0],
                'clips': [(c['best'], c['best_loss']) for c in clips]},
               out + '.%d' % rank)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharded_identification_equals_single_process(tmp_path):
    out = str(tmp_path / 'res')
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method='spawn')
    r = [torch.load(out + '.%d' % k, weights_only=False) for k in range(2)]
    # restarts 0..2 on rank 0, 3..4 on rank 1
    assert r[0]['range'] == (0, 3) and r[1]['range'] == (3, 5)
    assert r[0]['local'] == 3 and r[1]['local'] == 2
    # single process, same restarts
    orig_sim, orig_sync = identify.Simulator, torch.cuda.synchronize
    try:
        _setup_fakes()
        sc, tgt = _adam_case()
        ref = identify.adam_identify(sc, tgt, restarts=5, iters=40, lr=5e-2, free=(0, 2), seed=7,
                                     init_params=(0.5, 0.0, 1.0, 0.0))
        _setup_fakes(clip=True)
        sc2, tgt2, fpc = _clip_case()
        ref_clips = identify.clip_identify(sc2, tgt2, fpc, carry='full', restarts=3, iters=3, lr=1e-2, free=(0, 2))
    finally:
        identify.Simulator, torch.cuda.synchronize = orig_sim, orig_sync
    for k in range(2):
        np.testing.assert_array_equal(r[k]['best_params'], ref['best_params'])
        np.testing.assert_array_equal(r[k]['best_loss'], ref['best_loss'])
        np.testing.assert_array_equal(r[k]['history'], ref['history'])
        assert r[k]['best_index'] == ref['best_index']
        assert len(r[k]['clips']) == len(ref_clips) == 3
        for (b, l), c in zip(r[k]['clips'], ref_clips):
            np.testing.assert_array_equal(b, c['best'])
            assert l == c['best_loss']
