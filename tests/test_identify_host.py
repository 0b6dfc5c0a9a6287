"""The identification driver's host logic without a GPU: adam_identify
optimises in normalised coordinates inside the parameter box, keeps the best
parameters of every restart, and starts restart 0 from init_params;
clip_identify fits clip windows in order and carries the state (positions, or
the full state) from one clip's best-parameter rollout into the next;
export_profiles writes one x and one z profile per scene.  The
simulator is replaced by a differentiable stand-in whose force profile is
smooth in (K, n), so the driver itself is what is tested."""

import numpy as np
import pytest
import torch

from diffstir_gb300 import identify
from diffstir_gb300 import scene as S


class FakeSim:
    """Force profile f[t] = (K sin(w t) + n^2 cos(w t), 0, K n) per scene."""

    def __init__(self, scenes, max_steps, options=None):
        self.B = len(scenes) if isinstance(scenes, (list, tuple)) else 1
        self.device = torch.device('cpu')
        self.calls = 0

    def rollout(self, p, nsteps, ckpt_every=50):
        self.calls += 1
        t = torch.arange(nsteps, dtype=torch.float32).reshape(1, nsteps) * 0.05
        K, n = p[:, 0:1], p[:, 2:3]
        fx = K * torch.sin(t) + n * n * torch.cos(t)
        fz = (K * n).expand(-1, nsteps)
        return torch.stack([fx, torch.zeros_like(fx), fz], -1)

    def close(self):
        pass


@pytest.fixture
def fake(monkeypatch):
    monkeypatch.setattr(identify, 'Simulator', FakeSim)
    monkeypatch.setattr(torch.cuda, 'synchronize', lambda *a, **k: None)


def _target(truth, T):
    sim = FakeSim([None], T)
    p = torch.tensor([truth], dtype=torch.float32)
    return sim.rollout(p, T)[0].numpy()


def test_adam_recovers_parameters_inside_the_box(fake):
    T = 40
    sc = S.small_synthetic_scene(n_grid=8, ppc=1, n_steps=T, seed=0)
    truth = (1.2, 0.0, 0.7, 0.0)
    res = identify.adam_identify(sc, _target(truth, T), restarts=4, iters=300, lr=5e-2, free=(0, 2), seed=3)
    lo, hi = identify.HB_BOUNDS[0], identify.HB_BOUNDS[2]
    bp = res['best_params']
    assert np.all((bp[:, 0] >= lo[0] - 1e-6) & (bp[:, 0] <= lo[1] + 1e-6))
    assert np.all((bp[:, 2] >= hi[0] - 1e-6) & (bp[:, 2] <= hi[1] + 1e-6))
    best = res['best']
    assert abs(best[0] - truth[0]) < 0.02 * truth[0] and abs(best[2] - truth[2]) < 0.02 * truth[2], best
    assert res['history'].shape == (300, 4)
    assert np.all(res['best_loss'] <= res['history'].min(axis=0) + 1e-12)
    assert res['grad_evals'] == 1200 and res['sim'].calls == 300


def test_restart_zero_starts_from_init_params(fake):
    T = 20
    sc = S.small_synthetic_scene(n_grid=8, ppc=1, n_steps=T, seed=0)
    truth = (0.9, 0.0, 0.6, 0.0)
    seen = []
    identify.adam_identify(sc, _target(truth, T), restarts=3, iters=1, lr=1e-9, free=(0, 2), seed=1,
                           init_params=(0.5, 0.0, 1.0, 0.0), callback=lambda it, p, lv: seen.append(p.numpy()))
    p0 = seen[0][0]
    assert abs(p0[0] - 0.5) < 1e-5 and abs(p0[2] - 1.0) < 1e-5
    # unfitted parameters keep the scene's values; the other restarts are drawn
    assert np.allclose(seen[0][:, 1], sc.params[1]) and np.allclose(seen[0][:, 3], sc.params[3])
    assert not np.allclose(seen[0][1], seen[0][0])


class FakeClipSim(FakeSim):
    """FakeSim plus the state calls of clip_identify; every substep of a
    forward moves x by +0.001 in y and sets v to 1, so the carried state
    shows which clip produced it."""
    log = []

    def __init__(self, scenes, max_steps, options=None):
        super().__init__(scenes, max_steps, options)
        self.scene = scenes[0] if isinstance(scenes, (list, tuple)) else scenes
        self.n = self.scene.n_particles
        self.x = torch.as_tensor(self.scene.x0(), dtype=torch.float32).repeat(self.B, 1)
        self.v = torch.zeros_like(self.x)
        FakeClipSim.log.append(('create', self.B, float(self.scene.trajectory[0, 0])))

    def set_initial_state(self, x, v=None, C=None, F=None):
        self.x = torch.as_tensor(x, dtype=torch.float32).clone()
        self.v = torch.zeros_like(self.x) if v is None else torch.as_tensor(v, dtype=torch.float32).clone()
        FakeClipSim.log.append(('init', self.B, float(self.x[0, 1]), v is not None, C is not None))

    def set_params(self, p):
        pass

    def forward(self, nsteps, **kw):
        self.x[:, 1] += 0.001 * nsteps
        self.v[:] = 1.0
        return torch.zeros((self.B, nsteps, 3))

    def get_state(self):
        n = self.n
        return {'x': self.x[:n].clone(), 'v': self.v[:n].clone(), 'C': torch.zeros(n, 3, 3),
                'F': torch.eye(3).repeat(n, 1, 1)}

    def status(self):
        return 0


@pytest.mark.parametrize('carry', ['x', 'full'])
def test_clip_identify_windows_and_state_carry(monkeypatch, carry):
    monkeypatch.setattr(identify, 'Simulator', FakeClipSim)
    monkeypatch.setattr(torch.cuda, 'synchronize', lambda *a, **k: None)
    FakeClipSim.log = []
    T, fpc = 30, 10
    sc = S.small_synthetic_scene(n_grid=8, ppc=1, n_steps=T, seed=0)
    target = _target((1.0, 0.0, 0.7, 0.0), T)
    y0 = float(sc.x0()[0, 1])
    out = identify.clip_identify(sc, target, fpc, carry=carry, restarts=2, iters=2, lr=1e-2, free=(0, 2),
                                 first_clip_factor=3)
    assert [c['substeps'] for c in out] == [(0, 10), (10, 20), (20, 30)]
    assert [c['history'].shape[0] for c in out] == [6, 2, 2]
    # each clip's simulators see the trajectory window of that clip
    creates = [e for e in FakeClipSim.log if e[0] == 'create']
    starts = [float(sc.trajectory[t, 0]) for t in (0, 0, 10, 10, 20, 20)]
    assert [e[2] for e in creates] == pytest.approx(starts)
    # clip c > 0 starts from the state clip c-1's best-parameter rollout produced
    inits = [e for e in FakeClipSim.log if e[0] == 'init']
    assert len(inits) == 4  # clips 1 and 2: the batched fit and the roll-forward
    for k, clip in enumerate((1, 1, 2, 2)):
        assert inits[k][2] == pytest.approx(y0 + 0.001 * fpc * clip, abs=1e-5)
        assert inits[k][3] == (carry == 'full') and inits[k][4] == (carry == 'full')
    assert inits[0][1] == 2 and inits[1][1] == 1  # tiled over the restarts, then one scene


def test_export_profiles_writes_x_and_z_per_scene(tmp_path):
    from diffstir_gb300 import export

    class Sim:
        def forward(self, nsteps):
            f = torch.arange(2 * nsteps * 3, dtype=torch.float32).reshape(2, nsteps, 3)
            return f

    f = export.export_profiles(Sim(), 5, str(tmp_path), prefix='r_')
    for b in range(2):
        fx = np.load(str(tmp_path / ('r_force_profile_x_%d.npy' % b)))
        fz = np.load(str(tmp_path / ('r_force_profile_z_%d.npy' % b)))
        assert fx.dtype == np.float32 and fx.shape == (5,)
        np.testing.assert_array_equal(fx, f[b, :, 0])
        np.testing.assert_array_equal(fz, f[b, :, 2])
