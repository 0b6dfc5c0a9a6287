"""The reference-facing module (diffstir_gb300.compat) driven exactly as the
reference's callers drive src/simulator/simulation_functions.py, checked
against the FP64 oracle; the headless force export; the batched Adam
identification driver."""

import numpy as np
import pytest
import torch

import golden_util as gu
import oracle
from diffstir_gb300 import scene as S

pytestmark = pytest.mark.gpu


def _configure(n_frames=8, model=0):
    from diffstir_gb300 import compat as sf
    raw = S.reference_like_trajectory(n_frames)
    sf.configure(raw_trajectory=raw, seed=0, n_liquid=300, n_rod=40, n_container=60, n_grid=32)
    return sf


def _oracle_scene(sf):
    sc = sf._sc
    r = lambda a: np.asarray(a, np.float32).astype(np.float64)
    return sc.desc, r(sc.x0()), r(sc.trajectory)


def test_tape_epoch_matches_oracle():
    """One epoch of gradient_descent_module.parameters_fitting (:99-120)."""
    sf = _configure()
    params = (2.0, 0.1, 0.6, 0.8)
    target = np.random.default_rng(0).normal(0, 0.02, size=sf.max_steps)
    sf.initialize_objects()
    sf.model_index[None] = 0
    for j in range(4):
        sf.constitutive_parameters[j] = params[j]
    sf.operator_forces_seq.from_numpy(target)
    sf.initialize_ti_field()
    sf.loss[None] = 0
    with sf.ti.ad.Tape(loss=sf.loss):
        sf.loss[None] = 0
        for f in range(sf.max_steps - 1):
            sf.forward(f)
        sf.compute_loss()
    grad = np.array([sf.constitutive_parameters.grad[j] for j in range(4)])
    loss = sf.loss[None]
    desc, x0, traj = _oracle_scene(sf)
    desc.model = 0
    T = sf.max_steps - 1
    p = np.asarray(params, np.float32).astype(np.float64)
    force, _, _ = oracle.rollout(desc, p, traj, T, x0)
    loss_o, dF = gu.reference_loss_and_dforce(force, np.float32(target).astype(np.float64), T)
    _, dp_o, _, _ = oracle.grad(desc, p, traj, T, x0, dF)
    assert abs(loss - loss_o) <= 1e-4 * abs(loss_o)
    np.testing.assert_allclose(grad, dp_o, rtol=1e-3, atol=1e-3 * np.abs(dp_o).max())
    # positions of every frame are available like the reference's fields
    xs = sf.x.to_numpy()
    assert xs.shape == (sf.max_steps, 300, 3)
    _, states, _ = oracle.rollout(desc, p, traj, T, x0, return_states=True)
    np.testing.assert_allclose(xs[-1], states[T, :300, 0:3], atol=1e-5)
    # second epoch after initialize_ti_field reproduces the first
    sf.initialize_ti_field()
    sf.loss[None] = 0
    with sf.ti.ad.Tape(loss=sf.loss):
        sf.loss[None] = 0
        for f in range(sf.max_steps - 1):
            sf.forward(f)
        sf.compute_loss()
    grad2 = np.array([sf.constitutive_parameters.grad[j] for j in range(4)])
    np.testing.assert_allclose(grad2, grad, rtol=1e-4, atol=1e-6 * np.abs(grad).max())


def test_force_export_matches_oracle(tmp_path):
    from diffstir_gb300 import export
    sf = _configure(n_frames=10)
    sf.model_index[None] = 2
    for j, v in enumerate((0.8, 0.5, 0.7, 0.0)):
        sf.constitutive_parameters[j] = v
    out = export.force_calculation_and_export(str(tmp_path))
    fx = np.load(str(tmp_path / 'force_profile_x.npy'))
    assert fx.shape == (sf.max_steps,) and fx[0] == 0 and fx[-1] == 0
    desc, x0, traj = _oracle_scene(sf)
    desc.model = 2
    T = sf.max_steps - 1
    force, _, _ = oracle.rollout(desc, np.asarray((0.8, 0.5, 0.7, 0.0)), traj, T, x0)
    np.testing.assert_allclose(fx[1:T], force[:T - 1, 0], rtol=1e-3, atol=1e-4 * np.abs(force).max())
    assert out['stick_positions'].shape == (sf.max_steps - 1, 3)


def test_adam_identification_reduces_loss():
    from diffstir_gb300 import identify
    from diffstir_gb300.simulator import Simulator
    T = 60
    truth = np.array([0.8, 0.0, 0.7, 0.0])
    sc = S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=0, params=truth)
    sim = Simulator(sc, max_steps=T)
    target = sim.forward(T)[0].cpu().numpy()
    sc2 = S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=0, params=(1.0, 0.0, 0.9, 0.0))
    res = identify.adam_identify(sc2, target, restarts=4, iters=25, lr=5e-2, ckpt_every=10, free=(0, 2),
                                 bounds={0: (0.1, 2.0), 2: (0.4, 1.2)}, seed=1)
    h = res['history']
    assert np.all(np.isfinite(h))
    assert h[-1].min() < 0.5 * h[0].min()


def test_initial_state_continues_a_rollout():
    """A rollout restarted from the full state after substep 30 (through
    set_initial_state) reproduces substeps 30..59 of the continuous rollout:
    the state carry-over that clip-wise identification relies on."""
    from diffstir_gb300.scene import Scene
    from diffstir_gb300.simulator import Simulator
    T, h = 60, 30
    sc = S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=2)
    full = Simulator(sc, max_steps=T)
    f_full = full.forward(T)[0].cpu().numpy()
    first = Simulator(sc, max_steps=h)
    first.forward(h)
    st = first.get_state()
    n = sc.n_particles
    second_sc = Scene(sc.desc, sc.liquid_x, sc.rod_x, sc.container_x, sc.trajectory[h:], sc.params, dict(sc.info))
    second = Simulator(second_sc, max_steps=T - h)
    second.set_initial_state(st['x'], st['v'], st['C'].reshape(n, 9), st['F'].reshape(n, 9))
    f2 = second.forward(T - h)[0].cpu().numpy()
    ref = f_full[h:]
    assert np.abs(f2 - ref).max() <= 1e-4 * np.abs(ref).max()
    # reset() goes back to the carried state, not to x0
    second.reset()
    f3 = second.forward(T - h)[0].cpu().numpy()
    assert np.abs(f3 - ref).max() <= 1e-4 * np.abs(ref).max()
    for s_ in (full, first, second):
        s_.close()


def test_clip_identification_carries_state():
    from diffstir_gb300 import identify
    from diffstir_gb300.simulator import Simulator
    T, fpc = 60, 30
    truth = np.array([0.8, 0.0, 0.7, 0.0])
    sc = S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=0, params=truth)
    sim = Simulator(sc, max_steps=T)
    target = sim.forward(T)[0].cpu().numpy()
    sim.close()
    sc2 = S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=0, params=(1.0, 0.0, 0.9, 0.0))
    for carry in ('x', 'full'):
        res = identify.clip_identify(sc2, target, fpc, carry=carry, restarts=4, iters=8, lr=5e-2, ckpt_every=10,
                                     free=(0, 2), bounds={0: (0.1, 2.0), 2: (0.4, 1.2)}, seed=1,
                                     first_clip_factor=2)
        assert [r['clip'] for r in res] == [0, 1]
        assert [r['substeps'] for r in res] == [(0, 30), (30, 60)]
        assert res[0]['history'].shape == (16, 4) and res[1]['history'].shape == (8, 4)
        for r in res:
            assert r['status'] == 0 and np.isfinite(r['best_loss'])
        assert res[0]['best_loss'] < res[0]['history'][0].min()


@pytest.mark.gpu
def test_red_rate_probe_measures_a_positive_rate():
    """The vector-RED probe behind the scatter kernels' atomic roofline runs
    on the current stream and reports a plausible rate (sectors/s)."""
    import ctypes
    from diffstir_gb300 import _lib
    rate = ctypes.c_double(0.0)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert _lib.lib().dstir_measure_red_rate(1 << 18, 64, ctypes.byref(rate), s) == 0
    assert 1e9 < rate.value < 1e13, rate.value


@pytest.mark.gpu
def test_fp32_rate_probe_measures_a_plausible_rate():
    """The FP32 FMA probe behind the FP32 side of the roofline reports a rate
    between 1 and 1000 TFLOP/s."""
    import ctypes
    from diffstir_gb300 import _lib
    rate = ctypes.c_double(0.0)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert _lib.lib().dstir_measure_fp32_rate(2000, ctypes.byref(rate), s) == 0
    assert 1e12 < rate.value < 1e15, rate.value
