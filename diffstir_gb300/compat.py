"""Drop-in stand-in for the reference's simulator module.

The reference's callers (src/gradient_descent_module.py,
src/force_calculation_and_animation_module.py, main.py) do
``from src.simulator.simulation_functions import *`` and then drive module-level
Taichi kernels and fields.  This module exposes the same names with the same
meaning, backed by the GB300 simulator, so those callers run unchanged when
that import is redirected here, for instance by
``sys.modules['src.simulator.simulation_functions'] = diffstir_gb300.compat``
before the caller's own import runs::

    initialize_objects(), initialize_ti_field(), forward(f), backward(f),
    compute_loss(), ti.ad.Tape(loss=loss)
    loss[None], model_index[None], constitutive_parameters[j] (+ .grad[j]),
    learning_rate[j], parameters_lower_bound / parameters_upper_bound,
    x / operator_x / container_x / total_operator_dv .to_numpy(),
    initial_x / initial_operator_x / operator_kinematic_seq / operator_forces_seq .from_numpy(),
    max_steps, dt, dx, inv_dx, n_grid, bound, n_clips, frames_per_clip,
    operator_p_vol, operator_density, operator_p_mass, liquid_p_mass, ...

Semantics kept from the reference (src/simulator/simulation_functions.py):
* ``forward(f)`` advances substep f (:341-348); outside a tape it runs at once.
* ``compute_loss()`` adds each frame's rod dv into ``total_operator_dv`` and
  adds sum_f |F_x(f) - target(f)| / (max_steps-1) into ``loss`` (:330-339), so
  calling it twice accumulates twice, as in the reference.
* Inside ``ti.ad.Tape(loss=loss)`` the consecutive ``forward(f)`` calls are
  gathered into one checkpointed rollout; leaving the tape runs the adjoint and
  fills ``constitutive_parameters.grad`` (gradient_descent_module.py:103-120).
* Positions of every frame are kept on the GPU for ``to_numpy()``.

Configuration: :func:`configure` (config/arguments.json contents, trajectory
array, target forces, seed, particle counts); by default the reference
scene with the analytic stand-in trajectory.  The first use needs a CUDA GPU.
"""

import math
import types

import numpy as np

from . import scene as _scene

# ---------------------------------------------------------------------------
# configuration (initialization.py:14-70)
# ---------------------------------------------------------------------------
_cfg = {'args': None, 'raw_trajectory': None, 'force_magnitudes': None, 'seed': 0, 'n_liquid': None,
        'n_rod': None, 'n_container': None, 'n_grid': None, 'max_steps': None}
_state = types.SimpleNamespace(built=False)

dim = 3
bound = _scene.REFERENCE_BOUND
n_constitutive_parameters = 4
parameters_lower_bound = [0] * n_constitutive_parameters
parameters_upper_bound = [0] * n_constitutive_parameters


def configure(arguments=None, raw_trajectory=None, force_magnitudes=None, seed=0, n_liquid=None, n_rod=None,
              n_container=None, n_grid=None, max_steps=None):
    """Set the scene inputs the reference reads at import time
    (config/arguments.json, data/traj.npy, data/force.npy) and rebuild."""
    _cfg.update(args=arguments, raw_trajectory=raw_trajectory, force_magnitudes=force_magnitudes, seed=seed,
                n_liquid=n_liquid, n_rod=n_rod, n_container=n_container, n_grid=n_grid, max_steps=max_steps)
    _state.built = False
    _build_scene()


def _build_scene():
    g = globals()
    raw = _cfg['raw_trajectory']
    if raw is None:
        raw = _scene.reference_like_trajectory(_cfg['max_steps'] or 8000)
    raw = np.asarray(raw, dtype=np.float64)
    if _cfg['max_steps'] is not None:
        raw = raw[:_cfg['max_steps']]
    sc = _scene.reference_scene(seed=_cfg['seed'], raw_trajectory=raw, n_liquid=_cfg['n_liquid'],
                                n_rod=_cfg['n_rod'], n_container=_cfg['n_container'], n_grid=_cfg['n_grid'],
                                args=_cfg['args'])
    c = sc.info['constants']
    g['_sc'] = sc
    for k in ('dt', 'n_grid', 'dx', 'n_particles', 'n_container_particles', 'n_operator_particles',
              'uniform_scaling_factor', 'container_diameter', 'container_height', 'container_radius',
              'container_wall_thickness', 'liquid_height', 'operator_radius', 'operator_length',
              'liquid_density', 'operator_density', 'container_density', 'operator_bottom_height',
              'liquid_radius', 'operator_p_vol', 'liquid_p_vol', 'operator_p_mass', 'liquid_p_mass',
              'n_particles_container_wall', 'n_particles_container_bottom', 'container_p_vol',
              'container_p_mass'):
        g[k] = c[k]
    g['inv_dx'] = float(c['n_grid'])
    g['operator_mass'] = c['operator_p_mass'] * c['n_operator_particles']
    a = _cfg['args'] or _scene.REFERENCE_ARGUMENTS
    fpc = a['simulation_setting']['frames_per_clip']
    total_frames = raw.shape[0]
    if fpc >= total_frames:
        fpc = total_frames - 1
    g['frames_per_clip'] = fpc
    g['n_clips'] = int(total_frames / fpc)
    g['max_steps'] = total_frames
    g['n_simulation_frames'] = total_frames
    g['total_frames'] = total_frames
    g['operator_trajectory'] = sc.trajectory
    fm = _cfg['force_magnitudes']
    g['force_magnitudes'] = (np.zeros(total_frames) if fm is None else np.asarray(fm, dtype=np.float64))
    g['liquid_particles'] = sc.liquid_x
    g['operator_particles'] = sc.rod_x
    g['container_particles'] = sc.container_x
    _make_fields()
    _state.sim = None
    _state.built = True


# ---------------------------------------------------------------------------
# field wrappers
# ---------------------------------------------------------------------------
class _HostField:
    """A small field held on the host (scalars and parameter vectors)."""

    def __init__(self, shape, dtype=np.float32, with_grad=True):
        self._a = np.zeros(shape, dtype=dtype)
        self.grad = _HostField(shape, dtype, False) if with_grad else None

    def __getitem__(self, k):
        v = self._a[() if k is None else k]
        return v.item() if np.ndim(v) == 0 else v.copy()

    def __setitem__(self, k, v):
        self._a[() if k is None else k] = v

    def to_numpy(self):
        return self._a.copy()

    def from_numpy(self, arr):
        arr = np.asarray(arr)
        n = min(arr.shape[0], self._a.shape[0]) if self._a.ndim else None
        if n is None:
            self._a[()] = arr
        else:
            self._a[:n] = arr[:n]

    def fill(self, v):
        self._a[...] = v


class _InitialPositions:
    """initial_x / initial_operator_x / initial_container_x."""

    def __init__(self, kind):
        self.kind = kind

    def from_numpy(self, arr):
        arr = np.asarray(arr, dtype=np.float64).reshape(-1, 3)
        sc = _sc
        if self.kind == 0:
            sc.liquid_x = arr.copy()
        elif self.kind == 1:
            sc.rod_x = arr.copy()
        else:
            sc.container_x = arr.copy()
        if _state.sim is not None:
            _state.sim.set_x0(sc.x0())

    def to_numpy(self):
        sc = _sc
        return [sc.liquid_x, sc.rod_x, sc.container_x][self.kind].astype(np.float32)


class _Trajectory:
    """operator_kinematic_seq: frames of the rod reference point."""

    def from_numpy(self, arr):
        arr = np.asarray(arr, dtype=np.float64).reshape(-1, 3)
        t = _sc.trajectory.copy()
        n = min(arr.shape[0], t.shape[0])
        t[:n] = arr[:n]
        _sc.trajectory = t
        if _state.sim is not None:
            _state.sim.set_trajectories([t])

    def to_numpy(self):
        return _sc.trajectory.astype(np.float32)


class _PositionHistory:
    """x / operator_x / container_x: positions of every frame (read-only)."""

    def __init__(self, kind):
        self.kind = kind

    def to_numpy(self):
        _ensure_sim()
        _flush_pending(record=_state.tape is not None)
        _materialize_positions()
        h = _state.hist_x  # torch [max_steps, N, 3]
        sc = _sc
        nl, nr = sc.desc.n_liquid, sc.desc.n_rod
        sl = [slice(0, nl), slice(nl, nl + nr), slice(nl + nr, sc.n_particles)][self.kind]
        return h[:, sl].cpu().numpy()


class _TotalDv:
    def to_numpy(self):
        _flush_pending(record=_state.tape is not None)
        return _state.total_dv.copy()

    def __getitem__(self, k):
        return _state.total_dv[k].copy()


def _make_fields():
    g = globals()
    ms = g['max_steps']
    g['model_index'] = _HostField((), np.int32, False)
    g['constitutive_parameters'] = _HostField((n_constitutive_parameters,))
    g['learning_rate'] = _HostField((n_constitutive_parameters,), with_grad=False)
    g['loss'] = _HostField(())
    g['operator_forces_seq'] = _HostField((ms,), with_grad=False)
    g['operator_forces_seq'].from_numpy(g['force_magnitudes'])
    g['total_operator_dv'] = _TotalDv()
    g['initial_x'] = _InitialPositions(0)
    g['initial_operator_x'] = _InitialPositions(1)
    g['initial_container_x'] = _InitialPositions(2)
    g['operator_kinematic_seq'] = _Trajectory()
    g['x'] = _PositionHistory(0)
    g['operator_x'] = _PositionHistory(1)
    g['container_x'] = _PositionHistory(2)
    _state.total_dv = np.zeros((ms, 3), dtype=np.float32)
    _state.forces = {}          # frame f+1 -> force of substep f (numpy [3])
    _state.pending = []         # substeps gathered inside a tape
    _state.tape = None


def _ensure_sim():
    if _state.sim is None:
        import torch
        from .simulator import Simulator
        sim = Simulator(_sc, max_steps=max_steps - 1)
        _state.sim = sim
        _state.hist_x = torch.zeros((max_steps, sim.N, 3), device=sim.device)
        _state.hist_x[0] = sim.get_state()['x']
    return _state.sim


def _push_params():
    sim = _ensure_sim()
    p = constitutive_parameters.to_numpy()[None].astype(np.float32)
    sim.set_params(p, np.array([int(model_index[None])], dtype=np.int32))


# ---------------------------------------------------------------------------
# kernels of simulation_functions.py
# ---------------------------------------------------------------------------
def initialize_objects():
    """simulation_functions.py:293-298: upload the particles and trajectory, reset."""
    _ensure_sim().set_trajectories([_sc.trajectory])
    initialize_ti_field()


def initialize_ti_field():
    """simulation_functions.py:301-319: step-0 state, zero total_operator_dv."""
    sim = _ensure_sim()
    sim.reset()
    _state.hist_x[0] = sim.get_state()['x']
    _state.total_dv[...] = 0
    _state.forces = {}
    _state.pending = []
    _state.hist_pending = None


def forward(s):
    """One substep (simulation_functions.py:341-348).  Consecutive calls are
    gathered and run as one rollout when a result is needed (compute_loss,
    to_numpy, the end of a tape)."""
    s = int(s)
    if _state.pending and s != _state.pending[-1] + 1:
        _flush_pending(record=False)
    _state.pending.append(s)


def _flush_pending(record):
    if not _state.pending:
        return
    import torch
    sim = _ensure_sim()
    _push_params()
    t0, n = _state.pending[0], len(_state.pending)
    _state.pending = []
    if record:
        st0 = sim.get_state()
        force = sim.forward(n, t0=t0, ckpt_every=max(1, int(math.isqrt(n))), record=True)
        _state.rec = (t0, n)
        # positions of frames t0+1..t0+n are produced on demand (to_numpy) by
        # replaying from the saved start state on a second handle, so that the
        # recorded checkpoints of `sim` stay intact for the adjoint
        _state.hist_pending = (st0, t0, n, constitutive_parameters.to_numpy().copy(), int(model_index[None]),
                               _sc.trajectory.copy())
    else:
        _materialize_positions()
        force = torch.empty((1, n, 3), device=sim.device)
        for i in range(n):
            force[:, i] = sim.substep(t0 + i)
            _state.hist_x[t0 + i + 1] = sim.get_state()['x']
    fo = force[0].cpu().numpy()
    for i in range(n):
        _state.forces[t0 + i + 1] = fo[i]


def _materialize_positions():
    hp = getattr(_state, 'hist_pending', None)
    if hp is None:
        return
    from .simulator import Simulator
    st0, t0, n, prm, model, traj = hp
    if getattr(_state, 'shadow', None) is None:
        _state.shadow = Simulator(_sc, max_steps=max_steps - 1)
    sh = _state.shadow
    sh.set_trajectories([traj])
    sh.set_params(prm[None].astype(np.float32), np.array([model], dtype=np.int32))
    sh.set_state(st0['x'], st0['v'], st0['C'].reshape(-1, 9), st0['F'].reshape(-1, 9))
    for i in range(n):
        sh.substep(t0 + i)
        _state.hist_x[t0 + i + 1] = sh.get_state()['x']
    _state.hist_pending = None


def compute_loss():
    """simulation_functions.py:330-339."""
    _flush_pending(record=_state.tape is not None)
    T = max_steps - 1
    fs = np.float32(_sc.desc.force_scale)
    for step in range(T):
        if step in _state.forces:
            _state.total_dv[step] += _state.forces[step] / fs
    acc = _state.total_dv[:T] * np.float32(operator_p_vol * operator_density / dt)
    diff = acc[:, 0] - operator_forces_seq.to_numpy()[:T]
    loss[None] = loss[None] + float(np.abs(diff).sum() / T)
    _state.loss_diff = diff


def backward(s):
    """The reference's grad_for(forward) is run by the tape; calling it directly
    is not part of the callers' API (gradient_descent_module.py never does)."""
    raise RuntimeError('backward(s) runs inside ti.ad.Tape; use the tape')


class _Tape:
    """ti.ad.Tape(loss=loss): gathers forward(f) calls into one recorded,
    checkpointed rollout and runs the adjoint on exit."""

    def __init__(self, loss=None, clear_gradients=True):
        self.loss = loss
        self.clear = clear_gradients
        self.replaying = False

    def __enter__(self):
        if self.clear:
            constitutive_parameters.grad.fill(0)
        _flush_pending(record=False)
        _state.tape = self
        return self

    def __exit__(self, et, ev, tb):
        _state.tape = None
        if et is not None:
            return False
        if _state.pending:
            _flush_pending(record=True)
        import torch
        sim = _state.sim
        t0, n = _state.rec
        T = max_steps - 1
        # d loss / d F_x(frame) = sign(F_x - target) / (max_steps-1); frame f+1 <- substep f
        diff = _state.loss_diff
        dF = np.zeros((1, n, 3), dtype=np.float32)
        for i in range(n):
            frame = t0 + i + 1
            if frame < T:
                dF[0, i, 0] = np.sign(diff[frame]) / T
        dp = sim.backward(torch.from_numpy(dF).to(sim.device))
        g = constitutive_parameters.grad
        g._a[:] += dp[0].cpu().numpy()
        return False


ti = types.SimpleNamespace(ad=types.SimpleNamespace(Tape=_Tape), max=max, f32='f32', i32='i32')

_build_scene()
