"""Generate golden fixtures by executing the reference's own simulator source.

Test infrastructure.  Usage (in a container where the reference checkout is
present; the GPU machines never run this)::

    python tests/golden/make_golden.py /path/to/DiffStir-checkout

The reference (``src/simulator/simulation_functions.py`` and
``src/simulator/initialization.py``) is imported unmodified, with
``tests/golden/taichi_shim.py`` registered as ``taichi``.  Only its inputs are
replaced: the JSON read from ``config/arguments.json`` (smaller particle counts,
optionally another grid size), the trajectory array read from
``data/traj.npy`` (the first T+1 frames of the real one) and the force array.
NumPy's global RNG is seeded before import, so the reference's own rejection
sampler produces a reproducible scene.

For every fixture it records the scene the reference built, the rollout it
produced through ``forward(f)`` / ``compute_loss()``, and, under
``ti.ad.Tape(loss=loss)`` exactly as ``src/gradient_descent_module.py:103-107``
drives it, the gradients of the loss with respect to the constitutive
parameters and the step-0 particle state.
"""

import builtins
import io
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import taichi_shim  # noqa: E402

SF_NAMES = ('src', 'src.simulator', 'src.simulator.initialization',
            'src.simulator.simulation_functions')

# Parameter sets per model (reference order of constitutive_parameters):
#   0 Carreau [eta0, eta_inf, n, lambda]; 1 Cross [eta0, eta_inf, n, lambda];
#   2 Herschel-Bulkley [K, tau_y, n, unused]
MODEL_PARAMS = {
    0: [2.0, 0.1, 0.6, 0.8],
    1: [1.5, 0.2, 0.5, 1.2],
    2: [0.8, 0.5, 0.7, 0.0],
}


def load_reference(ref_root, cfg, traj, force, seed, prec):
    """Import the reference simulator with the given config/data contents."""
    for n in SF_NAMES:
        sys.modules.pop(n, None)
    taichi_shim._STATE.fields.clear()
    taichi_shim.set_precision(prec)
    taichi_shim.install()
    real_open, real_load = builtins.open, np.load

    def fake_open(path, *a, **kw):
        if str(path).endswith(os.path.join('config', 'arguments.json')):
            return io.StringIO(json.dumps(cfg))
        return real_open(path, *a, **kw)

    def fake_load(path, *a, **kw):
        p = str(path)
        if p.endswith('traj.npy'):
            return traj.copy()
        if p.endswith('force.npy'):
            return force.copy()
        return real_load(path, *a, **kw)

    np.random.seed(seed)
    builtins.open, np.load = fake_open, fake_load
    if ref_root not in sys.path:
        sys.path.insert(0, ref_root)
    try:
        import src.simulator.simulation_functions as sf  # noqa: F401
    finally:
        builtins.open, np.load = real_open, real_load
    sf.range = taichi_shim.shim_range
    return sf


def scene_record(sf):
    g = sf.__dict__
    keys = ['dt', 'n_grid', 'dx', 'inv_dx', 'bound', 'n_particles', 'n_operator_particles',
            'n_container_particles', 'uniform_scaling_factor', 'liquid_p_vol', 'liquid_p_mass',
            'operator_p_vol', 'operator_p_mass', 'operator_density', 'container_p_vol',
            'container_p_mass', 'max_steps', 'n_particles_container_wall',
            'n_particles_container_bottom']
    rec = {('scene_' + k): np.asarray(g[k], dtype=np.float64) for k in keys}
    rec['liquid_particles'] = np.asarray(g['liquid_particles'], dtype=np.float64)
    rec['operator_particles'] = np.asarray(g['operator_particles'], dtype=np.float64)
    rec['container_particles'] = np.asarray(g['container_particles'], dtype=np.float64)
    rec['operator_trajectory'] = np.asarray(g['operator_trajectory'], dtype=np.float64)
    return rec


STATE_KEYS = ('x', 'v', 'C', 'F', 'operator_x', 'operator_C', 'container_C')


def subsample_states(out, stride):
    """Keep the per-frame particle states of frames 0, stride, 2 stride, ...
    only (forces, losses and gradients stay complete); records the stride."""
    for key in list(out):
        if key[:1] == 'm' and key.split('_', 1)[-1] in STATE_KEYS:
            out[key] = out[key][::stride]
    out['meta_state_stride'] = np.int64(stride)


def run_fixture(ref_root, name, n_grid, n_liq, n_op, n_cont, T, seed, prec, models,
                with_grad, out_dir, extra=None):
    """``extra`` (optional): 'dt' replaces simulation_setting.dt, 'scene'
    updates scene_information, 'traj_quantum' rounds the trajectory to
    multiples of that power of two, so that the reference's centring
    (initialization.py:74-77) stays exact and the processed trajectory is
    exactly representable in float32: the rod velocity (q[f+1]-q[f])/dt
    (simulation_functions.py:266) then needs no float32 rounding of q, and a
    float32 simulator can be compared with this fixture directly."""
    extra = extra or {}
    cfg = json.load(open(os.path.join(ref_root, 'config', 'arguments.json')))
    ss = cfg['simulation_setting']
    ss['n_grid'] = n_grid
    ss['n_model_particles_generated'] = n_liq
    ss['n_operator_model_particles_generated'] = n_op
    ss['n_container_model_particles_generated'] = n_cont
    if 'dt' in extra:
        ss['dt'] = extra['dt']
    cfg['scene_information'].update(extra.get('scene', {}))
    traj_full = np.load(os.path.join(ref_root, 'data', 'traj.npy'))
    force_full = np.load(os.path.join(ref_root, 'data', 'force.npy'))
    traj = traj_full[:T + 1].copy()
    if 'traj_quantum' in extra:
        q = extra['traj_quantum']
        traj = np.round(traj / q) * q
    force = force_full[:T + 1].copy()
    rng = np.random.default_rng(1000 + seed)
    out = {}
    for model in models:
        t0 = time.time()
        sf = load_reference(ref_root, cfg, traj, force, seed, prec)
        if not out:
            out.update(scene_record(sf))
            out['raw_trajectory'] = traj.copy()
        params = MODEL_PARAMS[model]
        sf.model_index[None] = model
        for j in range(4):
            sf.constitutive_parameters[j] = params[j]
        # a target that straddles the simulated force so the L1 sign varies
        target = rng.normal(0.0, 0.02, size=sf.max_steps)
        sf.operator_forces_seq.from_numpy(target)
        sf.initialize_objects()
        sf.loss[None] = 0
        for f in range(sf.max_steps - 1):
            sf.forward(f)
        sf.compute_loss()
        p = 'm%d_' % model
        out[p + 'params'] = np.asarray(params, dtype=np.float64)
        out[p + 'target'] = target
        out[p + 'x'] = sf.x.to_numpy()
        out[p + 'v'] = sf.v.to_numpy()
        out[p + 'C'] = sf.C.to_numpy()
        out[p + 'F'] = sf.F.to_numpy()
        out[p + 'operator_x'] = sf.operator_x.to_numpy()
        out[p + 'operator_C'] = sf.operator_C.to_numpy()
        out[p + 'container_C'] = sf.container_C.to_numpy()
        out[p + 'operator_dv'] = sf.operator_dv.to_numpy()
        out[p + 'total_operator_dv'] = sf.total_operator_dv.to_numpy()
        out[p + 'loss'] = np.float64(sf.loss[None].v)
        if with_grad:
            sf.initialize_ti_field()
            sf.loss[None] = 0
            with taichi_shim.ad.Tape(loss=sf.loss):
                sf.loss[None] = 0
                for f in range(sf.max_steps - 1):
                    sf.forward(f)
                sf.compute_loss()
            out[p + 'loss_tape'] = np.float64(sf.loss[None].v)
            out[p + 'grad_params'] = sf.constitutive_parameters.grad.to_numpy()
            out[p + 'grad_x0'] = sf.x.grad.to_numpy()[0]
            out[p + 'grad_v0'] = sf.v.grad.to_numpy()[0]
            out[p + 'grad_F0'] = sf.F.grad.to_numpy()[0]
            out[p + 'grad_C1'] = sf.C.grad.to_numpy()[1] if sf.max_steps > 1 else np.zeros(0)
        print('%s model %d: %.1fs loss=%r' % (name, model, time.time() - t0,
                                               float(out[p + 'loss'])), flush=True)
    if 'state_stride' in extra:
        subsample_states(out, extra['state_stride'])
    out['meta_config'] = np.array(json.dumps(cfg))
    out['meta_prec'] = np.array(prec)
    out['meta_seed'] = np.int64(seed)
    out['meta_T'] = np.int64(T)
    path = os.path.join(out_dir, name + '.npz')
    np.savez_compressed(path, **out)
    print('wrote', path, os.path.getsize(path), 'bytes')


# Long fixtures: a wide, tall container on a 16^3 grid, so that within 60
# substeps at the reference's dt the fluid's nodes meet every boundary rule
# of grid_op (the container projection with mass :205-210, the six wall
# clamps :211-220 and the sticky top :221-224) and the rod dv (:266-270)
# accumulates over many frames.  Trajectory rounded to multiples of 2^-24.
LONG = {'scene': {'container_diameter': 0.74, 'liquid_height': 0.58, 'container_height': 0.6},
        'traj_quantum': 2.0 ** -24, 'state_stride': 10}

FIXTURES = {
    # name: (n_grid, n_liquid, n_rod, n_container, substeps T, seed, precision, models, grad[, extra])
    'ref_f64_g32': (32, 300, 40, 60, 6, 0, 'f64', (0, 1, 2), True),
    'ref_f32_g32': (32, 300, 40, 60, 6, 0, 'f32', (0, 1, 2), True),
    'ref_f64_g71': (71, 400, 50, 60, 3, 1, 'f64', (2,), True),
    'ref_f64_g16_long': (16, 160, 16, 40, 60, 0, 'f64', (0, 1, 2), True, LONG),
    'ref_f32_g16_long': (16, 160, 16, 40, 60, 0, 'f32', (0, 1, 2), True, LONG),
}


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else None
    assert ref_root and os.path.isdir(ref_root), 'pass the reference checkout path'
    names = sys.argv[2:] or list(FIXTURES)
    for name in names:
        args = FIXTURES[name]
        run_fixture(ref_root, name, *args[:9], out_dir=HERE, extra=args[9] if len(args) > 9 else None)


if __name__ == '__main__':
    main()
