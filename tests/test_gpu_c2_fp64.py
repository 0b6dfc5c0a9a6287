"""The 64^3 workload's gradient over its full horizon against FP64 (opt-in:
DIFFSTIR_SLOW=1; about ten minutes of host-core time for the FP64 oracle).

Workload: the 603,432-particle 64^3 scene of the benchmark (scene 0 of
configuration C2, 2000 substeps, checkpoint every 50, power-law fluid), loss
the mean squared error of the rod's x and z force profile against the profile
of seeded ground-truth parameters, as bench.py builds it.  The GPU's
checkpointed FP32 adjoint is compared with the FP64 oracle's adjoint (the
reverse pass of its own FP64 rollout, chained over 50-substep segments), and
both with FP64 central differences at h = 1e-3 x |param|.

After about 525 substeps the fluid reaches the top band, whose sticky rule
(simulation_functions.py:221-224) zeroes a node's whole velocity when v_y > 0:
the loss then jumps by small amounts as the parameters move, and central
differences pick those jumps up while the adjoint (the derivative of the
branch taken) does not.  So the FP64 differences sit a few 1e-3 from the FP64
adjoint; the GPU adjoint is held to the FP64 adjoint at 1e-4.
"""

import os

import numpy as np
import pytest
import torch

import oracle
from diffstir_gb300 import scene as S
from diffstir_gb300.simulator import Simulator

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get('DIFFSTIR_SLOW') != '1', reason='opt-in: DIFFSTIR_SLOW=1')]


def test_c2_full_horizon_gradient_vs_fp64():
    T, K = 2000, 50
    sc = S.synthetic_scene('C2', seed=0, n_steps=T)
    # target of seeded ground truth, as bench.py draws it for rank 0
    truth = S.draw_config_params('C2', np.random.default_rng(1000))
    sim = Simulator(sc, max_steps=T)
    sim.set_params(torch.tensor(truth[None], dtype=torch.float32, device='cuda'))
    sim.reset()
    target = sim.forward(T).clone()
    params = torch.tensor(sc.params[None], dtype=torch.float32, device='cuda')
    sim.set_params(params)
    sim.reset()
    f = sim.forward(T, ckpt_every=K, record=True)
    diff = (f - target)[..., 0::2]
    norm = float(diff.numel())
    dF = torch.zeros_like(f)
    dF[..., 0::2] = 2.0 * diff / norm
    dp_gpu = sim.backward(dF)[0].double().cpu().numpy()
    assert sim.status() == 0
    sim.close()

    threads = os.cpu_count() or 1
    x0 = np.asarray(sc.x0(), np.float32).astype(np.float64)
    traj = np.asarray(sc.trajectory, np.float32).astype(np.float64)
    p = np.asarray(params[0].cpu().numpy(), np.float64)
    tgt = target[0].double().cpu().numpy()
    f64 = oracle.rollout_chain(sc.desc, p, traj, T, x0, K, threads)
    w = np.zeros((T, 3))
    w[:, 0::2] = 2.0 * (f64 - tgt)[:, 0::2] / norm
    _, dp64 = oracle.rollout_chain(sc.desc, p, traj, T, x0, K, threads, w)

    def loss(pp):
        ff = oracle.rollout_chain(sc.desc, pp, traj, T, x0, K, threads)
        d = (ff - tgt)[:, 0::2]
        return float((d * d).sum() / norm)

    report = {}
    for i, name in ((0, 'K'), (2, 'n')):
        h = 1e-3 * abs(p[i])
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (loss(pp) - loss(pm)) / (2.0 * h)
        report[name] = (dp_gpu[i], dp64[i], fd)
        assert abs(dp_gpu[i] - dp64[i]) <= 1e-4 * abs(dp64[i]), (name, dp_gpu[i], dp64[i])
        assert abs(dp64[i] - fd) <= 1e-2 * abs(fd), (name, dp64[i], fd)
    print('C2 2000 substeps: (GPU adjoint, FP64 adjoint, FP64 central difference h=1e-3):', report)
