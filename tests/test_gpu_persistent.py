"""Persistent segment launches (option "persist").

For small scenes a substep is bound by launch latency: P2G, the grid update
and G2P (and their adjoints) are each a launch of a few dozen blocks.  With
"persist" every chunk of a forward chain and every segment of the reverse
pass runs as one cooperative launch, its phases separated by grid-wide
barriers.  These tests check (1) that the persistent path gives the
per-launch path's forces, gradients and step-0 state adjoints, for a batch of
uneven scenes over several re-sorted checkpoint segments, with and without
graph replay, and (2) the bounded wait: with "barrier_test" every barrier
waits for one arrival that never comes, so each wait runs out after
"barrier_limit_us", the launch stops early and raises DSTIR_STATUS_TIMEOUT in
the status word; the context stays usable and the next launches are right.
"""

import numpy as np
import pytest
import torch

from diffstir_gb300 import _abi
from diffstir_gb300 import scene as S
from diffstir_gb300.simulator import Simulator

from test_gpu_parity import rel, rounded

pytestmark = pytest.mark.gpu


def _scenes(T):
    return [rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=21)),
            rounded(S.small_synthetic_scene(n_grid=20, ppc=4, n_steps=T, seed=22, hi=(0.7, 0.45, 0.7),
                                            params=(2.0, 0.1, 0.6, 0.8), model=S.MODEL_CARREAU))]


def _run(scenes, T, K, wts, opts, reps=2):
    sim = Simulator(scenes, max_steps=T, options=opts)
    out = []
    for _ in range(reps):
        sim.reset()
        f = sim.forward(T, ckpt_every=K, record=True).cpu().numpy()
        dp, ds = sim.backward(torch.as_tensor(wts, dtype=torch.float32, device='cuda'), want_state0=True)
        out.append((f, dp.cpu().numpy(), {k: v.cpu().numpy() for k, v in ds.items()}))
    st = sim.status()
    active = sim.get_option('persist_active')
    sim.close()
    return out, st, active


@pytest.mark.parametrize('graph', [0, 1])
def test_persistent_matches_per_launch_path(graph):
    T, K = 34, 7
    scenes = _scenes(T)
    wts = np.random.default_rng(9).normal(size=(2, T, 3))
    ref, st0, act0 = _run(scenes, T, K, wts, {'p2g': 1, 'graph': graph})
    got, st1, act1 = _run(scenes, T, K, wts, {'p2g': 1, 'graph': graph, 'persist': 1})
    assert st0 == 0 and st1 == 0
    assert act0 == 0 and act1 == 1
    f0, dp0, ds0 = ref[0]
    for f, dp, ds in got:
        assert rel(f, f0) < 1e-5
        assert rel(dp, dp0) < 1e-4
        for k in 'xvCF':
            assert rel(ds[k], ds0[k]) < 1e-3, k


def test_persistent_long_chunks_split_into_several_launches():
    # 120 substeps in one segment: the forward chain and the segment's reverse
    # pass run as three persistent launches each (at most 50 substeps apiece)
    T = 120
    sc = rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=23))
    wts = np.random.default_rng(10).normal(size=(1, T, 3))
    ref, _, _ = _run([sc], T, T, wts, {'p2g': 1}, reps=1)
    got, st, act = _run([sc], T, T, wts, {'p2g': 1, 'persist': 1}, reps=1)
    assert st == 0 and act == 1
    assert rel(got[0][0], ref[0][0]) < 1e-5
    assert rel(got[0][1], ref[0][1]) < 1e-4


def test_barrier_wait_runs_out_and_reports_timeout():
    T = 6
    sc = rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=24))
    sim = Simulator(sc, max_steps=T, options={'p2g': 1, 'persist': 1, 'graph': 0})
    f_ok = sim.forward(T).cpu().numpy()
    assert sim.status() == 0
    # every barrier now waits for an arrival that nothing makes; 20 ms limit
    sim.set_option('barrier_limit_us', 20000)
    sim.set_option('barrier_test', 1)
    sim.reset()
    sim.forward(T)
    torch.cuda.synchronize()
    assert sim.status() & _abi.DSTIR_STATUS_TIMEOUT
    # the reverse pass's launches time out the same way
    sim.reset()
    f = sim.forward(T, ckpt_every=3, record=True)
    sim.backward(torch.ones_like(f))
    torch.cuda.synchronize()
    assert sim.status() & _abi.DSTIR_STATUS_TIMEOUT
    # back to normal barriers: the context is usable and the results right
    sim.set_option('barrier_test', 0)
    sim.reset()
    f2 = sim.forward(T).cpu().numpy()
    assert sim.status() == 0
    assert rel(f2, f_ok) < 1e-5
    sim.close()
