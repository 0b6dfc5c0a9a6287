"""Parity at the benchmark sizes, over a short horizon.

The 64^3 single-scene workload (603k particles) and the 128^3 workload
(~4.8M particles, sinusoid rod path) run a few substeps on the GPU and on the
FP64 oracle (OpenMP on the host cores) from the same float32-rounded inputs:
rod force within 1e-4 relative and parameter gradient within 1e-3 relative,
for the default configuration and the brick-tiled one.  A batch of three
full-size scenes must reproduce each scene run alone.
"""

import os

import numpy as np
import pytest
import torch

import oracle
from diffstir_gb300 import scene as S
from diffstir_gb300.scene import Scene
from diffstir_gb300.simulator import Simulator

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def rounded(sc):
    return Scene(sc.desc, f32(sc.liquid_x), f32(sc.rod_x), f32(sc.container_x), f32(sc.trajectory),
                 f32(sc.params), dict(sc.info))


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-30))


@pytest.mark.parametrize('config,T', [('C2', 6), ('C4', 3)])
@pytest.mark.parametrize('opts', [{'p2g': 1}, {'p2g': 3}, {'p2g': 4}], ids=['vec', 'brick', 'warp'])
def test_full_size_force_and_gradient(config, T, opts):
    sc = rounded(S.synthetic_scene(config, seed=0, n_steps=T))
    wts = np.random.default_rng(0).normal(size=(T, 3))
    sim = Simulator(sc, max_steps=T, options=opts)
    force = sim.forward(T, ckpt_every=2, record=True)
    dp = sim.backward(torch.as_tensor(wts[None], dtype=torch.float32, device='cuda'))
    torch.cuda.synchronize()
    assert sim.status() == 0
    f_o, dp_o, _, st = oracle.grad(sc.desc, sc.params, sc.trajectory, T, sc.x0(), wts, threads=THREADS)
    assert st == 0
    assert rel(force[0].cpu().numpy(), f_o) < 1e-4
    idx = [0, 2] if sc.params[1] == 0 else [0, 1, 2]
    assert rel(dp[0].cpu().numpy()[idx], dp_o[idx]) < 1e-3
    sim.close()


def test_full_size_batch_equals_single():
    T = 4
    scenes = [rounded(S.synthetic_scene('C3', seed=s, n_steps=T)) for s in range(3)]
    wts = np.random.default_rng(1).normal(size=(3, T, 3))
    sim = Simulator(scenes, max_steps=T, options={'p2g': 3})
    fb = sim.forward(T, ckpt_every=2, record=True).cpu().numpy()
    gb = sim.backward(torch.as_tensor(wts, dtype=torch.float32, device='cuda')).cpu().numpy()
    sim.close()
    for b, sc in enumerate(scenes):
        s1 = Simulator(sc, max_steps=T, options={'p2g': 3})
        f1 = s1.forward(T, ckpt_every=2, record=True).cpu().numpy()
        g1 = s1.backward(torch.as_tensor(wts[b:b + 1], dtype=torch.float32, device='cuda')).cpu().numpy()
        s1.close()
        assert rel(fb[b], f1[0]) < 1e-5
        assert rel(gb[b], g1[0]) < 1e-4


def test_full_size_gravity_only_substep():
    """Rod-free, stress-free first substep of the full 64^3 scene: only gravity
    acts, so the binned scatter and gather must give every particle zero
    horizontal velocity and a vertical one between dt*g and 0 (walls and the
    1e-10 mass floor at sparse surface nodes only shrink it), with the bulk of
    the particles at exactly dt*g (the B-spline weights sum to one)."""
    sc = rounded(S.synthetic_scene('C2', seed=0, n_steps=1))
    sc.desc.rod_radius = 0.0
    sc.desc.bulk_modulus = 0.0
    sim = Simulator(sc, max_steps=1, options={'p2g': 3})
    sim.forward(1)
    v = sim.get_state()['v'].cpu().numpy()
    sim.close()
    g = sc.desc.dt * sc.desc.gravity
    np.testing.assert_allclose(v[:, 0], 0.0, atol=1e-9)
    np.testing.assert_allclose(v[:, 2], 0.0, atol=1e-9)
    assert np.all(v[:, 1] <= 0.0) and np.all(v[:, 1] >= g * (1 + 1e-5))
    assert abs(np.median(v[:, 1]) - g) < 1e-4 * abs(g)   # 1e-10 mass floor / ~4e-6 node mass


def test_c1_full_length_gradient_vs_fp64_differences():
    """The 32^3 workload over its full 500 substeps: the GPU adjoint of the
    force-MSE loss against central differences (h = 1e-3 x |param|) of the
    FP64 oracle's loss, for K and n; within 1e-3 relative.  The GPU rollout is
    FP32 throughout, so this bounds rounding drift over the whole horizon as
    well as the adjoint itself."""
    T = 500
    sc = rounded(S.synthetic_scene('C1', seed=0, n_steps=T))
    truth = np.array([0.5, 0.0, 0.7, 0.0])
    f_t, _, st = oracle.rollout(sc.desc, truth, sc.trajectory, T, sc.x0(), precision='f64', threads=THREADS)
    assert st == 0
    p = np.array([0.8, 0.0, 0.9, 0.0])

    def oracle_loss(pp):
        f, _, s_ = oracle.rollout(sc.desc, pp, sc.trajectory, T, sc.x0(), precision='f64', threads=THREADS)
        assert s_ == 0
        d = (f - f_t)[:, 0::2]
        return (d * d).sum() / d.size

    sim = Simulator(sc, max_steps=T)
    sim.set_params(torch.tensor(p[None], dtype=torch.float32, device='cuda'))
    sim.reset()
    f = sim.forward(T, ckpt_every=50, record=True)[0].double().cpu().numpy()
    d = (f - f_t)[:, 0::2]
    w = np.zeros((1, T, 3))
    w[0, :, 0::2] = 2.0 * d / d.size
    dp = sim.backward(torch.as_tensor(w, dtype=torch.float32, device='cuda'))[0].cpu().numpy()
    assert sim.status() == 0
    sim.close()
    for i in (0, 2):
        h = 1e-3 * abs(p[i])
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (oracle_loss(pp) - oracle_loss(pm)) / (2 * h)
        assert abs(dp[i] - fd) <= 1e-3 * abs(fd), (i, dp[i], fd)


def test_long_horizon_adjoint_matches_fp64_adjoint_with_top_band_contact():
    """The 64^3 workload's block and parameters at 32^3 over 600 substeps, by
    which time the fluid has reached the top band where the reference's sticky
    top makes the loss jump in the parameters.  Difference quotients are then
    no reference for the pointwise derivative, but the FP64 oracle's adjoint
    is: the GPU adjoint (FP32 throughout, re-sorted particle order, 50-substep
    checkpoints) matches it within 1e-3 relative."""
    cfg = S.CONFIGS['C2']
    p = f32([0.11404720693826675, 0.0, 0.8690828084945679, 0.0])
    truth = f32(S.draw_config_params('C2', np.random.default_rng(1000)))
    pos = f32(S.block_particles(32, 8, cfg['lo'], cfg['hi'], np.random.default_rng(0)))
    desc = S.synthetic_desc(32, 8, pos.shape[0], dt=cfg['dt'], rod_radius=cfg['rod_radius'])
    T = 600
    z = np.zeros((0, 3))
    sc = Scene(desc, pos, z, z, f32(S.circle_trajectory(T, cfg['dt'])), p, {})
    ft, _, st = oracle.rollout(desc, truth, sc.trajectory, T, pos, threads=THREADS)
    assert st == 0
    f_o, _, _ = oracle.rollout(desc, p, sc.trajectory, T, pos, threads=THREADS)
    d = (f_o - ft)[:, 0::2]
    w = np.zeros((T, 3))
    w[:, 0::2] = 2.0 * d / d.size
    _, dp_o, _, st = oracle.grad(desc, p, sc.trajectory, T, pos, w, threads=THREADS)
    assert st == 0
    sim = Simulator(sc, max_steps=T)
    sim.set_params(torch.tensor(p[None], dtype=torch.float32, device='cuda'))
    sim.reset()
    sim.forward(T, ckpt_every=50, record=True)
    dp = sim.backward(torch.as_tensor(w[None], dtype=torch.float32, device='cuda'))[0].cpu().numpy()
    assert sim.status() == 0
    sim.close()
    assert rel(dp[[0, 2]], dp_o[[0, 2]]) < 1e-3, (dp, dp_o)
