"""Headless force-profile export, the non-graphical part of
force_calculation_and_animation (src/force_calculation_and_animation_module.py:3-21,54-56).

The reference runs the rollout, saves the rod force profiles
``force_profile_x.npy`` / ``force_profile_z.npy`` (frames, float32) and the
liquid point clouds / rod centre positions, then opens an Open3D window.  The
window is unavailable on this machine (no graphics stack); the arrays it would show
are written instead.
"""

import os

import numpy as np


def force_calculation_and_export(out_dir, presentation_time=None):
    """Same steps as the reference function, through :mod:`diffstir_gb300.compat`
    (configure it first).  Returns the dict of arrays written."""
    from . import compat as sf
    os.makedirs(out_dir, exist_ok=True)
    if presentation_time is None:
        presentation_time = (sf.max_steps - 1) * sf.dt
    sf.initialize_objects()
    sf.loss[None] = 0
    for f in range(int(presentation_time / sf.dt - 1)):
        sf.forward(f)
    sf.compute_loss()
    pos_series = sf.x.to_numpy()
    operator_pos_series = sf.operator_x.to_numpy()
    total = sf.total_operator_dv.to_numpy() * sf.operator_p_vol * sf.operator_density / sf.dt
    out = {
        'force_profile_x': total[:, 0].astype(np.float32),
        'force_profile_z': total[:, 2].astype(np.float32),
        'liquid_point_clouds': pos_series.astype(np.float32),
        'stick_positions': np.mean(operator_pos_series, axis=1)[:-1].astype(np.float32),
    }
    for k, v in out.items():
        np.save(os.path.join(out_dir, k + '.npy'), v)
    out['loss'] = float(sf.loss[None])
    return out


def export_profiles(sim, nsteps, out_dir, prefix=''):
    """Force profiles of a :class:`~diffstir_gb300.simulator.Simulator` rollout
    ([B, nsteps, 3], entry f = force of substep f) saved per scene."""
    os.makedirs(out_dir, exist_ok=True)
    f = sim.forward(nsteps).cpu().numpy()
    for b in range(f.shape[0]):
        np.save(os.path.join(out_dir, '%sforce_profile_x_%d.npy' % (prefix, b)), f[b, :, 0].astype(np.float32))
        np.save(os.path.join(out_dir, '%sforce_profile_z_%d.npy' % (prefix, b)), f[b, :, 2].astype(np.float32))
    return f
