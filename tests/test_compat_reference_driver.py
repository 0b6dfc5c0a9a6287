"""The reference's own identification driver against the drop-in module.

src/gradient_descent_module.py of the reference is imported UNMODIFIED, with
``src.simulator.simulation_functions`` (the Taichi module it star-imports)
aliased to diffstir_gb300.compat, and its parameters_fitting (the epoch loop
of :84-139: ti.ad.Tape over forward(f) and compute_loss, then the reference's
magnitude-scaled step rule single_parameter_fitting1) runs to the end of its
first clip.  This test runs without a GPU: the simulator under compat is
replaced by a stand-in that executes the FP64 CPU oracle through the same
methods compat calls (set_params, forward(record=True), backward, substep,
get_state, ...).  What it checks is the drop-in boundary itself: every name
the driver uses exists with the reference's meaning, the tape gathers the
substeps into one recorded rollout and fills constitutive_parameters.grad
with the gradient of the reference's L1 force loss, and the losses the driver
records are the oracle's.  The reference checkout is read at run time, so
the test is skipped where it is absent (the GPU machines)."""

import importlib.util
import os
import sys
import types

import numpy as np
import pytest
import torch

import oracle
from diffstir_gb300 import compat
from diffstir_gb300 import simulator as simmod

REF = os.environ.get('DIFFSTIR_REFERENCE', '/root/reference')
DRIVER = os.path.join(REF, 'src', 'gradient_descent_module.py')


class OracleSim:
    """CPU stand-in of simulator.Simulator for one scene, backed by the FP64
    oracle (test infrastructure)."""

    def __init__(self, scene, max_steps=None, **kw):
        self.sc = scene
        self.N = scene.n_particles
        self.B = 1
        self.max_steps = max_steps
        self.device = torch.device('cpu')
        self.traj = np.asarray(scene.trajectory, np.float64)
        self.params = np.asarray(scene.params, np.float64)
        self.model = scene.desc.model
        self._x0 = scene.x0()
        self.reset()

    def _desc(self):
        d = type(self.sc.desc)()
        import ctypes
        ctypes.memmove(ctypes.byref(d), ctypes.byref(self.sc.desc), ctypes.sizeof(d))
        d.model = int(self.model)
        return d

    def set_trajectories(self, trajs):
        self.traj = np.asarray(trajs[0], np.float64)

    def set_x0(self, x0):
        self._x0 = np.asarray(x0, np.float64).reshape(self.N, 3)

    def reset(self):
        self.st = np.zeros((self.N, 24))
        self.st[:, 0:3] = self._x0
        self.st[:, 15:24] = np.eye(3).reshape(1, 9)

    def set_state(self, x, v=None, C=None, F=None):
        self.st = np.zeros((self.N, 24))
        self.st[:, 0:3] = np.asarray(x).reshape(self.N, 3)
        if v is not None:
            self.st[:, 3:6] = np.asarray(v).reshape(self.N, 3)
        if C is not None:
            self.st[:, 6:15] = np.asarray(C).reshape(self.N, 9)
        self.st[:, 15:24] = np.eye(3).reshape(1, 9) if F is None else np.asarray(F).reshape(self.N, 9)

    def get_state(self):
        t = torch.from_numpy(self.st.astype(np.float32))
        return {'x': t[:, 0:3], 'v': t[:, 3:6], 'C': t[:, 6:15].reshape(-1, 3, 3), 'F': t[:, 15:24].reshape(-1, 3, 3)}

    def set_params(self, p, models=None):
        self.params = np.asarray(p, np.float64).reshape(4)
        if models is not None:
            self.model = int(np.asarray(models).reshape(-1)[0])

    def _roll(self, t0, n):
        s = self.st
        f, last, _ = oracle.rollout_last(self._desc(), self.params, self.traj[t0:t0 + n + 1], n, s[:, 0:3], s[:, 3:6],
                                         s[:, 6:15], s[:, 15:24])
        return f, last

    def forward(self, n, t0=0, ckpt_every=50, record=False):
        if record:
            self.rec = (t0, n, self.st.copy(), self.params.copy(), self.model)
        f, self.st = self._roll(t0, n)
        return torch.from_numpy(f[None].astype(np.float32))

    def substep(self, f):
        frc, self.st = self._roll(f, 1)
        return torch.from_numpy(frc.astype(np.float32))

    def backward(self, dF):
        t0, n, s, prm, model = self.rec
        cur = (self.params, self.model)
        self.params, self.model = prm, model
        _, dp, _, _ = oracle.grad(self._desc(), prm, self.traj[t0:t0 + n + 1], n, s[:, 0:3],
                                  np.asarray(dF, np.float64).reshape(n, 3), s[:, 3:6], s[:, 6:15], s[:, 15:24])
        self.params, self.model = cur
        return torch.from_numpy(dp[None].astype(np.float32))


def _load_driver():
    pkg = types.ModuleType('src')
    pkg.__path__ = [os.path.join(REF, 'src')]
    sub = types.ModuleType('src.simulator')
    sub.__path__ = [os.path.join(REF, 'src', 'simulator')]
    saved = {k: sys.modules.get(k) for k in ('src', 'src.simulator', 'src.simulator.simulation_functions',
                                             'src.gradient_descent_module')}
    sys.modules.update({'src': pkg, 'src.simulator': sub, 'src.simulator.simulation_functions': compat})
    try:
        spec = importlib.util.spec_from_file_location('src.gradient_descent_module', DRIVER)
        mod = importlib.util.module_from_spec(spec)
        sys.modules['src.gradient_descent_module'] = mod
        spec.loader.exec_module(mod)
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return mod


@pytest.mark.skipif(not os.path.exists(DRIVER), reason='reference checkout not present')
def test_reference_parameters_fitting_runs_unmodified_against_compat(monkeypatch):
    monkeypatch.setattr(simmod, 'Simulator', OracleSim)
    raw = np.load(os.path.join(REF, 'data', 'traj.npy'))[:21]
    compat.configure(raw_trajectory=raw, seed=3, n_liquid=150, n_rod=16, n_container=40, n_grid=16)
    try:
        drv = _load_driver()
        # driven as main.py drives it (main.py:9-16): model and starting parameters
        compat.model_index[None] = 2
        for j, v in enumerate((0.8, 0.5, 0.7, 0.0)):
            compat.constitutive_parameters[j] = v
            compat.parameters_lower_bound[j] = 0.0
            compat.parameters_upper_bound[j] = 10.0
        target = np.random.default_rng(4).normal(0.0, 0.02, size=compat.max_steps)
        compat.operator_forces_seq.from_numpy(target)

        seen = []
        real_tape = compat._Tape

        class SpyTape(real_tape):
            def __exit__(self, et, ev, tb):
                p = compat.constitutive_parameters.to_numpy().copy()
                r = super().__exit__(et, ev, tb)
                seen.append((p, float(compat.loss[None]), compat.constitutive_parameters.grad.to_numpy().copy()))
                return r

        monkeypatch.setattr(compat.ti.ad, 'Tape', SpyTape)
        sc = compat._sc
        T = compat.max_steps - 1
        desc = OracleSim(sc)._desc()
        desc.model = 2                         # model_index[None] of the run
        # the clip's end moves the initial positions to the last frame
        # (initial_x.from_numpy, gradient_descent_module.py:131-132): keep the start
        x0, traj = sc.x0().copy(), sc.trajectory.copy()
        best = drv.parameters_fitting(1)       # clip 0 runs 3 epochs
        assert not np.allclose(sc.x0(), x0)
    finally:
        compat.configure()                     # back to the default scene
    assert len(seen) == 3 and len(best) == 4
    for p, loss, grad in seen:
        # the oracle's own L1 loss and its gradient at the parameters of that epoch
        f, _, _ = oracle.rollout(desc, p.astype(np.float64), traj, T, x0)
        acc = np.concatenate([[0.0], f[:T - 1, 0]])
        diff = acc - target[:T].astype(np.float32)   # operator_forces_seq holds float32
        assert abs(loss - np.abs(diff).sum() / T) <= 1e-5 * abs(loss)
        dF = np.zeros((T, 3))
        dF[:T - 1, 0] = np.sign(diff[1:]) / T
        _, dp, _, _ = oracle.grad(desc, p.astype(np.float64), traj, T, x0, dF)
        np.testing.assert_allclose(grad, dp, rtol=1e-5, atol=1e-9 * np.abs(dp).max())
    # the driver returns the parameters of its best epoch
    losses = [l for _, l, _ in seen]
    np.testing.assert_allclose(best, seen[int(np.argmin(losses))][0], rtol=1e-6)
