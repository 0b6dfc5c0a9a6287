"""The identification driver's host logic without a GPU: adam_identify
optimises in normalised coordinates inside the parameter box, keeps the best
parameters of every restart, and starts restart 0 from init_params.  The
simulator is replaced by a differentiable stand-in whose force profile is
smooth in (K, n), so the optimiser itself is what is tested."""

import numpy as np
import pytest
import torch

from diffstir_gb300 import identify
from diffstir_gb300 import scene as S


class FakeSim:
    """Force profile f[t] = (K sin(w t) + n^2 cos(w t), 0, K n) per scene."""

    def __init__(self, scenes, max_steps, options=None):
        self.B = len(scenes)
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
