"""GPU parity: the CUDA path (through the C ABI) against the FP64 CPU oracle.

Inputs are rounded to float32 before they reach either side, so the comparison
isolates arithmetic.  Bars: rod force profile within 1e-4 relative, parameter
gradients within 1e-3 relative (relative to the largest entry), as stated for
the path; states within 1e-4 relative.
"""

import os

import numpy as np
import pytest
import torch

import golden_util as gu
import oracle
from diffstir_gb300 import scene as S
from diffstir_gb300.scene import Scene
from diffstir_gb300.simulator import Simulator

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-4
GRAD_RTOL = 1e-3


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def rounded(sc):
    """Copy of a scene with every input rounded to float32."""
    return Scene(sc.desc, f32(sc.liquid_x), f32(sc.rod_x), f32(sc.container_x), f32(sc.trajectory),
                 f32(sc.params), dict(sc.info))


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def gpu_force_and_grad(sc, T, wts, ckpt=50, options=None, want_state0=False):
    sim = Simulator(sc, max_steps=T, options=options)
    force = sim.forward(T, ckpt_every=ckpt, record=True)
    out = sim.backward(torch.as_tensor(wts[None], dtype=torch.float32, device='cuda'), want_state0=want_state0)
    torch.cuda.synchronize()
    st = sim.status()
    if want_state0:
        dp, ds = out
        return force[0].cpu().numpy(), dp[0].cpu().numpy(), {k: v.cpu().numpy() for k, v in ds.items()}, st
    return force[0].cpu().numpy(), out[0].cpu().numpy(), None, st


def oracle_force_and_grad(sc, T, wts, want_state0=False):
    _, dp, ds, st = oracle.grad(sc.desc, sc.params, sc.trajectory, T, sc.x0(), wts, want_state0=want_state0)
    force, _, _ = oracle.rollout(sc.desc, sc.params, sc.trajectory, T, sc.x0())
    return force, dp, ds


def fixture_scene(name, model):
    d = gu.load(name)
    desc = gu.desc_from_fixture(d, model)
    return Scene(desc, d['liquid_particles'], d['operator_particles'], d['container_particles'],
                 d['operator_trajectory'], d['m%d_params' % model]), d


VARIANTS = [{'p2g': 1, 'fuse': 1, 'fuse_adj': 1}, {'p2g': 1}, {'p2g': 1, 'fuse': 1, 'fuse_adj': 0},
            {'p2g': 0, 'fuse': 1, 'fuse_adj': 1, 'graph': 1}, {'p2g': 3},
            {'p2g': 3, 'brick_scatter': 0}, {'p2g': 3, 'brick_scatter': 2}, {'p2g': 3, 'brick_gather': 0},
            {'p2g': 3, 'graph': 1}, {'p2g': 4}, {'p2g': 4, 'fuse': 1, 'fuse_adj': 1}, {'p2g': 4, 'resort': 0},
            {'p2g': 4, 'graph': 1}, {'p2g': 4, 'tight': 0}, {'p2g': 4, 'tight': 1},
            {'p2g': 4, 'fuse': 1, 'fuse_adj': 1, 'tight': 0}, {'p2g': 4, 'store_grids': 1},
            {'p2g': 4, 'store_grids': 1, 'graph': 1}, {'p2g': 4, 'lsort': 0},
            {'p2g': 4, 'block': 128}, {'p2g': 4, 'block': 64, 'graph': 1}, {'p2g': 4, 'pdl': 0},
            {'p2g': 4, 'fuse': 1, 'fuse_adj': 1, 'graph': 1}, {'p2g': 4, 'pdl': 2, 'graph': 1},
            {'p2g': 4, 'lstage': 0}, {'p2g': 4, 'graph': 1, 'block': 128, 'tight': 2}, {'p2g': 4, 'graph': 0},
            {'p2g': 1, 'persist': 1, 'graph': 0}, {'p2g': 1, 'persist': 1, 'graph': 1},
            {'p2g': 1, 'persist': 1, 'store_grids': 1}, {'p2g': 4, 'gprio': 0, 'graph': 1}]
VARIANT_IDS = ['vec-fused', 'vec-unfused', 'vec-fwdfused', 'plain-fused-graph', 'brick-red', 'brick-atom',
               'brick-global', 'brick-nogather', 'brick-graph', 'warp', 'warp-fused', 'warp-nosort', 'warp-graph',
               'warp-tight0', 'warp-tight1', 'warp-fused-tight0', 'warp-store', 'warp-store-graph', 'warp-nolsort',
               'warp-block128', 'warp-block64-graph', 'warp-nopdl', 'warp-fused-graph', 'warp-pdl2-graph',
               'warp-nostage', 'warp-graph-block128-tight2', 'warp-eager', 'vec-persist', 'vec-persist-graph',
               'vec-persist-store', 'warp-noprio-graph']


@pytest.mark.parametrize('opts', VARIANTS, ids=VARIANT_IDS)
@pytest.mark.parametrize('model', [0, 1, 2])
def test_reference_scene_golden(model, opts):
    """The reference's scene (container, rod particles, k=20000) as the
    reference's own code built and ran it for 60 substeps, in a wide, tall
    container whose fluid meets every wall clamp, the sticky top and the
    container projection (tests/golden/make_golden.py, fixture
    ref_f64_g16_long).  The GPU is compared directly with the reference's own
    results: its rod force profile (compute_loss, simulation_functions.py
    :330-339) within 1e-4 and the gradient of its L1 loss that ti.ad.Tape
    produced (gradient_descent_module.py:103-107) within 1e-3, given the same
    dL/dforce; and with the FP64 oracle on the same inputs.  The fixture's
    trajectory is exactly representable in float32, so the rod velocity
    (q[f+1]-q[f])/dt is the same on both sides."""
    sc, d = fixture_scene('ref_f64_g16_long', model)
    T = sc.n_steps
    p = 'm%d_' % model
    # the reference's force (compute_loss :335-336, in float64); entry f+1 is the GPU's entry f
    scale = float(d['scene_operator_p_vol']) * float(d['scene_operator_density']) / float(d['scene_dt'])
    ref_force = d[p + 'total_operator_dv'] * scale
    loss, dF = gu.reference_loss_and_dforce(ref_force[1:], d[p + 'target'], T)
    assert abs(loss - float(d[p + "loss"])) <= 1e-10 * abs(loss)
    force_g, dp_g, _, st = gpu_force_and_grad(sc, T, dF, ckpt=25, options=opts)
    assert st == 0
    assert rel(force_g[:T - 1], ref_force[1:T]) < FORCE_RTOL
    assert rel(dp_g, d[p + 'grad_params']) < GRAD_RTOL, (dp_g, d[p + 'grad_params'])
    scr = rounded(sc)
    force_o, dp_o, _ = oracle_force_and_grad(scr, T, dF)
    assert rel(force_g, force_o) < FORCE_RTOL
    assert rel(dp_g, dp_o) < GRAD_RTOL, (dp_g, dp_o)


@pytest.mark.parametrize('model', [0, 1, 2])
def test_reference_scene_golden_g32(model):
    """The 32^3 fixture (6 substeps): GPU against the FP64 oracle on
    float32-rounded inputs.  Its trajectory is not float32-exact, so the
    direct comparison with the reference's own numbers is the oracle's
    (tests/test_oracle_golden.py), not this one's."""
    sc, d = fixture_scene('ref_f64_g32', model)
    sc = rounded(sc)
    T = sc.n_steps
    force_o, _, _ = oracle.rollout(sc.desc, sc.params, sc.trajectory, T, sc.x0())
    loss, dF = gu.reference_loss_and_dforce(force_o, d['m%d_target' % model], T)
    force_g, dp_g, _, st = gpu_force_and_grad(sc, T, dF)
    assert st == 0
    _, dp_o, _ = oracle_force_and_grad(sc, T, dF)
    assert rel(force_g, force_o) < FORCE_RTOL
    assert rel(dp_g, dp_o) < GRAD_RTOL, (dp_g, dp_o)


@pytest.mark.parametrize('model,params', [(S.MODEL_HB, (0.5, 0.3, 0.7, 0.0)),
                                          (S.MODEL_CARREAU, (2.0, 0.1, 0.6, 0.8)),
                                          (S.MODEL_CROSS, (1.5, 0.2, 0.5, 1.2))])
@pytest.mark.parametrize('j_mode', [S.J_DET, S.J_SVD])
@pytest.mark.parametrize('opts', VARIANTS, ids=VARIANT_IDS)
def test_cylinder_scene_parity(model, params, j_mode, opts):
    T = 40
    sc = rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, params=params, model=model,
                                         j_mode=j_mode, seed=1))
    wts = np.random.default_rng(0).normal(size=(T, 3))
    force_g, dp_g, ds_g, st = gpu_force_and_grad(sc, T, wts, ckpt=7, want_state0=True, options=opts)
    assert st == 0
    force_o, dp_o, ds_o = oracle_force_and_grad(sc, T, wts, want_state0=True)
    assert rel(force_g, force_o) < FORCE_RTOL
    idx = [0, 1, 2] if model == S.MODEL_HB else [0, 1, 2, 3]
    assert rel(dp_g[idx], dp_o[idx]) < GRAD_RTOL, (dp_g, dp_o)
    assert rel(ds_g['x'], ds_o[:, 0:3]) < 1e-2
    assert rel(ds_g['F'].reshape(-1, 9), ds_o[:, 15:24]) < 1e-2


@pytest.mark.parametrize('opts', [{'p2g': 4}, {'p2g': 4, 'graph': 1, 'tight': 2}, {'p2g': 1, 'lsort': 0}],
                         ids=['warp', 'warp-graph-tight2', 'vec'])
def test_state_adjoint_dot_product_vs_fp64(opts):
    """Dot-product test of the GPU reverse pass against FP64: for a random
    direction u over all 24 components of a step-0 state with nonzero v, C
    and F - I, <J^T w, u> from the GPU adjoint (re-sorted segments) equals
    <w, J u> from central differences of the FP64 oracle along u."""
    T, K = 24, 6
    sc = rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=14))
    rng = np.random.default_rng(15)
    wts = rng.normal(size=(T, 3))
    x0 = sc.x0()
    n = x0.shape[0]
    v0 = rng.normal(scale=0.05, size=(n, 3)).astype(np.float32).astype(np.float64)
    C0 = rng.normal(scale=0.2, size=(n, 9)).astype(np.float32).astype(np.float64)
    F0 = (np.tile(np.eye(3).reshape(1, 9), (n, 1)) + rng.normal(scale=0.01, size=(n, 9))).astype(np.float32)
    F0 = F0.astype(np.float64)
    sim = Simulator(sc, max_steps=T, options=opts)
    sim.set_initial_state(*(torch.as_tensor(a, dtype=torch.float32, device='cuda') for a in (x0, v0, C0, F0)))
    sim.forward(T, ckpt_every=K, record=True)
    _, ds = sim.backward(torch.as_tensor(wts[None], dtype=torch.float32, device='cuda'), want_state0=True)
    assert sim.status() == 0
    g = np.concatenate([ds['x'].cpu().numpy().reshape(n, 3), ds['v'].cpu().numpy().reshape(n, 3),
                        ds['C'].cpu().numpy().reshape(n, 9), ds['F'].cpu().numpy().reshape(n, 9)], 1)
    sim.close()
    u = rng.normal(size=(n, 24))
    u[:, :3] *= 1e-2
    h = 1e-6

    def proj(sign):
        f, _, _ = oracle.rollout(sc.desc, sc.params, sc.trajectory, T, x0 + sign * h * u[:, :3],
                                 v0 + sign * h * u[:, 3:6], C0 + sign * h * u[:, 6:15], F0 + sign * h * u[:, 15:])
        return float((wts * f).sum())

    jvp = (proj(1) - proj(-1)) / (2 * h)
    vjp = float((g * u).sum())
    assert abs(vjp - jvp) <= 2e-4 * abs(jvp), (vjp, jvp)  # FP32 oracle on the CPU: 2e-6


def test_forward_states_match_oracle():
    T = 30
    sc = rounded(S.small_synthetic_scene(n_grid=16, ppc=4, n_steps=T, seed=2))
    sim = Simulator(sc, max_steps=T)
    sim.forward(T)
    st = sim.get_state()
    _, states, _ = oracle.rollout(sc.desc, sc.params, sc.trajectory, T, sc.x0(), return_states=True)
    last = states[T]
    assert rel(st['x'].cpu().numpy(), last[:, 0:3]) < 1e-5
    assert rel(st['v'].cpu().numpy(), last[:, 3:6]) < 1e-3
    assert rel(st['C'].cpu().numpy().reshape(-1, 9), last[:, 6:15]) < 1e-3
    assert rel(st['F'].cpu().numpy().reshape(-1, 9), last[:, 15:24]) < 1e-4


def test_forward_states_match_oracle_after_resorts():
    """A rollout re-sorted every 7 substeps returns its state in the caller's
    particle order."""
    T = 30
    sc = rounded(S.small_synthetic_scene(n_grid=16, ppc=4, n_steps=T, seed=2))
    sim = Simulator(sc, max_steps=T, options={'p2g': 4})
    sim.forward(T, ckpt_every=7)
    st = sim.get_state()
    _, states, _ = oracle.rollout(sc.desc, sc.params, sc.trajectory, T, sc.x0(), return_states=True)
    last = states[T]
    assert rel(st['x'].cpu().numpy(), last[:, 0:3]) < 1e-5
    assert rel(st['v'].cpu().numpy(), last[:, 3:6]) < 1e-3
    assert rel(st['F'].cpu().numpy().reshape(-1, 9), last[:, 15:24]) < 1e-4


@pytest.mark.parametrize('opts', [{'p2g': 1}, {'p2g': 4}, {'p2g': 4, 'fuse': 1, 'fuse_adj': 1},
                                  {'p2g': 4, 'graph': 1}], ids=['vec', 'warp', 'warp-fused', 'warp-graph'])
def test_resort_matches_fixed_order(opts):
    """Re-sorting the particles at every checkpoint changes only the order of
    the float atomics: forces, final state, parameter gradient and the
    adjoint of the step-0 state (in the caller's order) match the run without
    re-sort.  Two scenes of different sizes, ten segments, twice in a row."""
    T, K = 40, 4
    scenes = [rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=6)),
              rounded(S.small_synthetic_scene(n_grid=20, ppc=4, n_steps=T, seed=7))]
    wts = torch.as_tensor(np.random.default_rng(4).normal(size=(2, T, 3)), dtype=torch.float32, device='cuda')
    out = {}
    for rs in (0, 1):
        sim = Simulator(scenes, max_steps=T, options=dict(opts, resort=rs))
        for rep in range(2):
            sim.reset()
            f = sim.forward(T, ckpt_every=K, record=True).cpu().numpy()
            st = {k: v.cpu().numpy() for k, v in sim.get_state().items()}
            dp, ds = sim.backward(wts, want_state0=True)
            out[(rs, rep)] = (f, st, dp.cpu().numpy(), {k: v.cpu().numpy() for k, v in ds.items()})
        assert sim.status() == 0
        sim.close()
    f0, st0, dp0, ds0 = out[(0, 0)]
    for key in ((0, 1), (1, 0), (1, 1)):
        f, st, dp, ds = out[key]
        assert rel(f, f0) < 1e-5
        for k in 'xvCF':
            assert rel(st[k], st0[k]) < 1e-4, k
        assert rel(dp, dp0) < 1e-4
        for k in 'xvCF':
            assert rel(ds[k], ds0[k]) < 1e-3, k


@pytest.mark.parametrize('block', [256, 128, 64])
@pytest.mark.parametrize('lstage', [0, 1])
def test_local_interleave_matches_block_order(block, lstage):
    """Rebuilding the interleaved order inside each block before the warp
    scatters (option lsort) only changes which lane handles which particle:
    forces, final state, parameter gradient and the adjoint of the step-0
    state match the run in block order.  Two scenes of 8 particles per cell
    (full and partial blocks), long segments so that the particles drift far
    from the re-sorted order."""
    T, K = 60, 30
    scenes = [rounded(S.small_synthetic_scene(n_grid=24, ppc=8, n_steps=T, seed=12)),
              rounded(S.small_synthetic_scene(n_grid=20, ppc=4, n_steps=T, seed=13))]
    wts = torch.as_tensor(np.random.default_rng(6).normal(size=(2, T, 3)), dtype=torch.float32, device='cuda')
    out = {}
    for ls in (0, 1):
        sim = Simulator(scenes, max_steps=T, options={'p2g': 4, 'lsort': ls, 'block': block, 'lstage': lstage})
        assert sim.get_option('lsort') == ls
        sim.reset()
        f = sim.forward(T, ckpt_every=K, record=True).cpu().numpy()
        st = {k: v.cpu().numpy() for k, v in sim.get_state().items()}
        dp, ds = sim.backward(wts, want_state0=True)
        out[ls] = (f, st, dp.cpu().numpy(), {k: v.cpu().numpy() for k, v in ds.items()})
        assert sim.status() == 0
        sim.close()
    f0, st0, dp0, ds0 = out[0]
    f, st, dp, ds = out[1]
    assert rel(f, f0) < 1e-5
    for k in 'xvCF':
        assert rel(st[k], st0[k]) < 1e-4, k
    assert rel(dp, dp0) < 1e-4
    for k in 'xvCF':
        assert rel(ds[k], ds0[k]) < 1e-3, k


@pytest.mark.parametrize('opts', [{'p2g': 1}, {'p2g': 4}, {'p2g': 4, 'fuse': 1, 'fuse_adj': 1}, {'p2g': 0},
                                  {'p2g': 4, 'graph': 1}], ids=['vec', 'warp', 'warp-fused', 'plain', 'warp-graph'])
def test_box_skip_matches_full_grid(opts):
    """Skipping the grid nodes outside each scene's occupied box leaves
    forces, state and gradients as with the full grid update; two scenes of
    different sizes, the second one re-sorted at every checkpoint."""
    T, K = 36, 6
    scenes = [rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=8)),
              rounded(S.small_synthetic_scene(n_grid=24, ppc=4, n_steps=T, seed=9))]
    wts = torch.as_tensor(np.random.default_rng(5).normal(size=(2, T, 3)), dtype=torch.float32, device='cuda')
    out = {}
    for box in (0, 1):
        sim = Simulator(scenes, max_steps=T, options=dict(opts, box=box))
        f = sim.forward(T, ckpt_every=K, record=True).cpu().numpy()
        st = {k: v.cpu().numpy() for k, v in sim.get_state().items()}
        dp, ds = sim.backward(wts, want_state0=True)
        assert sim.status() == 0
        fs = sim.substep(T - 1).cpu().numpy()   # the single-substep entry point too
        out[box] = (f, st, dp.cpu().numpy(), {k: v.cpu().numpy() for k, v in ds.items()}, fs)
        sim.close()
    f0, st0, dp0, ds0, fs0 = out[0]
    f1, st1, dp1, ds1, fs1 = out[1]
    assert rel(f1, f0) < 1e-5
    for k in 'xvCF':
        assert rel(st1[k], st0[k]) < 1e-4, k
        assert rel(ds1[k], ds0[k]) < 1e-3, k
    assert rel(dp1, dp0) < 1e-4
    assert rel(fs1, fs0) < 1e-4


@pytest.mark.parametrize('opts', [{'p2g': 4}, {'p2g': 1, 'graph': 1}, {'p2g': 4, 'resort': 0}, {'p2g': 0}],
                         ids=['warp', 'vec-graph', 'warp-noresort', 'plain'])
def test_kept_grids_match_recompute(opts):
    """Keeping every substep's P2G and velocity grids (the reverse pass then
    recomputes states with G2P alone) gives the forces, gradients and
    step-0 state adjoint of the full segment recompute; two scenes, twice."""
    T, K = 30, 8
    scenes = [rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=12)),
              rounded(S.small_synthetic_scene(n_grid=20, ppc=4, n_steps=T, seed=13))]
    wts = torch.as_tensor(np.random.default_rng(7).normal(size=(2, T, 3)), dtype=torch.float32, device='cuda')
    out = {}
    for keep in (0, 1):
        sim = Simulator(scenes, max_steps=T, options=dict(opts, store_grids=keep))
        for rep in range(2):
            sim.reset()
            f = sim.forward(T, ckpt_every=K, record=True).cpu().numpy()
            dp, ds = sim.backward(wts, want_state0=True)
            out[(keep, rep)] = (f, dp.cpu().numpy(), {k: v.cpu().numpy() for k, v in ds.items()})
        assert sim.status() == 0
        sim.close()
    f0, dp0, ds0 = out[(0, 0)]
    for key in ((0, 1), (1, 0), (1, 1)):
        f, dp, ds = out[key]
        assert rel(f, f0) < 1e-5
        assert rel(dp, dp0) < 1e-4
        for k in 'xvCF':
            assert rel(ds[k], ds0[k]) < 1e-3, k


@pytest.mark.parametrize('opts', [{'p2g': 4}, {'p2g': 4, 'graph': 1}, {'p2g': 4, 'store_grids': 1},
                                  {'p2g': 4, 'fuse': 1, 'fuse_adj': 1}, {'p2g': 0, 'resort': 0}],
                         ids=['warp', 'warp-graph', 'warp-kept', 'warp-fused', 'plain'])
def test_overlapped_reverse_pass_matches_serial(opts):
    """The reverse pass with the segment recompute on a second stream
    (overlapping the adjoint of the next segment) gives the serial pass's
    forces, gradients and step-0 state adjoint; two scenes, seven segments,
    twice in a row."""
    T, K = 34, 5
    scenes = [rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=14)),
              rounded(S.small_synthetic_scene(n_grid=20, ppc=4, n_steps=T, seed=15))]
    wts = torch.as_tensor(np.random.default_rng(8).normal(size=(2, T, 3)), dtype=torch.float32, device='cuda')
    out = {}
    for ovl in (0, 1):
        sim = Simulator(scenes, max_steps=T, options=dict(opts, overlap=ovl))
        for rep in range(2):
            sim.reset()
            f = sim.forward(T, ckpt_every=K, record=True).cpu().numpy()
            dp, ds = sim.backward(wts, want_state0=True)
            out[(ovl, rep)] = (f, dp.cpu().numpy(), {k: v.cpu().numpy() for k, v in ds.items()})
        assert sim.status() == 0
        sim.close()
    f0, dp0, ds0 = out[(0, 0)]
    for key in ((0, 1), (1, 0), (1, 1)):
        f, dp, ds = out[key]
        assert rel(f, f0) < 1e-5
        assert rel(dp, dp0) < 1e-4
        for k in 'xvCF':
            assert rel(ds[k], ds0[k]) < 1e-3, k


def test_checkpoint_interval_invariance():
    T = 24
    sc = rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=4))
    wts = np.random.default_rng(3).normal(size=(T, 3))
    grads = [gpu_force_and_grad(sc, T, wts, ckpt=k)[1] for k in (1, 5, 24)]
    for g in grads[1:]:
        assert rel(g, grads[0]) < 1e-4


def test_p2g_variants_agree():
    T = 20
    sc = rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=5))
    wts = np.random.default_rng(4).normal(size=(T, 3))
    f0, g0, _, _ = gpu_force_and_grad(sc, T, wts, options={'p2g': 0})
    for opts in ({'p2g': 1}, {'p2g': 4}, {'p2g': 4, 'block': 128, 'gblock': 128}, {'p2g': 1, 'graph': 1},
                 {'p2g': 3}, {'p2g': 3, 'block': 64, 'gblock': 128}):
        f1, g1, _, _ = gpu_force_and_grad(sc, T, wts, options=opts)
        assert rel(f1, f0) < 1e-5, opts
        assert rel(g1, g0) < 1e-4, opts


def test_graph_replay_matches_eager_and_is_reusable():
    T = 18
    sc = rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=7))
    wts = torch.as_tensor(np.random.default_rng(8).normal(size=(1, T, 3)), dtype=torch.float32, device='cuda')
    eager = Simulator(sc, max_steps=T, options={'p2g': 3, 'graph': 0})
    graph = Simulator(sc, max_steps=T, options={'p2g': 3, 'graph': 1})
    fe = eager.forward(T, ckpt_every=5, record=True)
    ge = eager.backward(wts)
    for rep in range(3):  # replays of the cached graphs with new parameters
        p = torch.tensor(sc.params[None] * (1 + 0.1 * rep), dtype=torch.float32, device='cuda')
        for sim in (eager, graph):
            sim.set_params(p)
            sim.reset()
        fe = eager.forward(T, ckpt_every=5, record=True)
        ge = eager.backward(wts)
        fg = graph.forward(T, ckpt_every=5, record=True)
        gg = graph.backward(wts)
        torch.cuda.synchronize()
        assert rel(fg.cpu().numpy(), fe.cpu().numpy()) < 1e-5
        assert rel(gg.cpu().numpy(), ge.cpu().numpy()) < 1e-4
    # the launch counter counts the kernels inside each replayed graph
    for sim in (eager, graph):
        sim.reset()
        sim.set_option('launches', 0)
        sim.forward(T, ckpt_every=5, record=True)
        sim.backward(wts)
    assert graph.get_option('launches') == eager.get_option('launches') > 0


def test_batched_equals_single():
    """Scenes of uneven size and different parameters/models in one handle give
    the per-scene results."""
    T = 20
    scenes = [rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=s, hi=(0.7, h, 0.7),
                                              params=p, model=m))
              for s, h, p, m in ((0, 0.30, (0.5, 0.0, 0.7, 0.0), S.MODEL_HB),
                                 (1, 0.42, (2.0, 0.1, 0.6, 0.8), S.MODEL_CARREAU),
                                 (2, 0.22, (0.9, 0.4, 0.8, 0.0), S.MODEL_HB))]
    wts = np.random.default_rng(5).normal(size=(len(scenes), T, 3))
    for opts in ({'p2g': 1}, {'p2g': 3, 'graph': 1}, {'p2g': 4}):
        sim = Simulator(scenes, max_steps=T, options=opts)
        force = sim.forward(T, ckpt_every=6, record=True).cpu().numpy()
        dp = sim.backward(torch.as_tensor(wts, dtype=torch.float32, device='cuda')).cpu().numpy()
        for b, sc in enumerate(scenes):
            f1, g1, _, _ = gpu_force_and_grad(sc, T, wts[b], ckpt=6)
            assert rel(force[b], f1) < 1e-5
            assert rel(dp[b], g1) < 1e-4


def test_reference_scene_rod_particles_71():
    path = os.path.join(gu.GOLDEN_DIR, 'ref_f64_g71.npz')
    if not os.path.exists(path):
        pytest.skip('fixture not generated')
    sc, d = fixture_scene('ref_f64_g71', 2)
    sc = rounded(sc)
    T = sc.n_steps
    force_o, _, _ = oracle.rollout(sc.desc, sc.params, sc.trajectory, T, sc.x0())
    _, dF = gu.reference_loss_and_dforce(force_o, d['m2_target'], T)
    force_g, dp_g, _, _ = gpu_force_and_grad(sc, T, dF)
    _, dp_o, _ = oracle_force_and_grad(sc, T, dF)
    assert rel(force_g, force_o) < FORCE_RTOL
    assert rel(dp_g, dp_o) < GRAD_RTOL


def test_autograd_function_matches_backward():
    T = 16
    sc = rounded(S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=6))
    sim = Simulator(sc, max_steps=T)
    params = torch.tensor(sc.params[None], dtype=torch.float32, device='cuda', requires_grad=True)
    target = torch.zeros((1, T, 3), device='cuda')
    force = sim.rollout(params, ckpt_every=4)
    loss = ((force[..., [0, 2]] - target[..., [0, 2]]) ** 2).mean()
    loss.backward()
    wts = (2 * force.detach() / (T * 2)).cpu().numpy()[0]
    wts[:, 1] = 0
    _, dp, _, _ = gpu_force_and_grad(sc, T, wts, ckpt=4)
    assert rel(params.grad[0].cpu().numpy(), dp) < 1e-4


def test_svd_kernels_match_oracle():
    from diffstir_gb300 import ops
    rng = np.random.default_rng(0)
    A = rng.normal(size=(512, 3, 3)).astype(np.float32)
    A[:128] = (np.eye(3) + 0.05 * rng.normal(size=(128, 3, 3))).astype(np.float32)
    U, Sg, V = ops.svd3(torch.from_numpy(A).cuda())
    U, Sg, V = U.cpu().numpy(), Sg.cpu().numpy(), V.cpu().numpy()
    rec = np.einsum('nij,nj,nkj->nik', U, Sg, V)
    np.testing.assert_allclose(rec, A, atol=2e-5 * np.abs(A).max())
    assert np.all(np.linalg.det(U) > 0) and np.all(np.linalg.det(V) > 0)
    np.testing.assert_allclose(np.abs(Sg), np.linalg.svd(A.astype(np.float64), compute_uv=False), rtol=1e-4,
                               atol=1e-5)
    gU, gS, gV = (rng.normal(size=(512, 3, 3)), rng.normal(size=(512, 3)), rng.normal(size=(512, 3, 3)))
    Uo, So, Vo = oracle.svd3(A.astype(np.float64))
    gA_o = oracle.svd3_backward(gU, gS, gV, Uo, So, Vo)
    t = lambda a: torch.as_tensor(np.asarray(a, np.float32)).cuda()
    gA = ops.svd3_backward(t(gU), t(gS), t(gV), t(Uo), t(So), t(Vo)).cpu().numpy()
    err = np.abs(gA - gA_o).max(axis=(1, 2)) / np.maximum(np.abs(gA_o).max(axis=(1, 2)), 1.0)
    assert np.median(err) < 1e-4 and np.max(err) < 1e-2


@pytest.mark.parametrize('opts', VARIANTS, ids=VARIANT_IDS)
def test_out_of_grid_particle_sets_status_and_is_skipped(opts):
    T = 4
    sc = S.small_synthetic_scene(n_grid=16, ppc=1, n_steps=T, seed=0)
    x = sc.x0()
    x[0] = (-0.5, 0.5, 0.5)   # base < 0
    x[1] = (2.0, 0.5, 0.5)    # base > n-3
    sc.liquid_x = x
    sim = Simulator(sc, max_steps=T, options=opts)
    sim.forward(T, record=True, ckpt_every=2)
    sim.backward(torch.ones((1, T, 3), device='cuda'))
    torch.cuda.synchronize()
    flags = sim.status()
    assert flags & 2
    st = sim.get_state()
    assert torch.isfinite(st['x'][2:]).all()
