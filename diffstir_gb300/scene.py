"""Scene construction: the reference scene and the synthetic benchmark scenes.

A :class:`Scene` bundles one ``DstirSceneDesc`` (constants of the simulation,
include/diffstir.h), its particle positions ``[liquid | rod | container]``, the
rod trajectory and the constitutive parameters.

* :func:`reference_scene` restates src/simulator/initialization.py:14-117 of
  the reference: the derived constants (:21-54), the trajectory preparation
  (:74-78) and the rejection sampler of the container, liquid and rod
  particles (:79-117).  The reference samples with NumPy's global RNG and no
  seed; here the same calls, in the same order, are made on a seeded
  ``RandomState`` so that ``seed=s`` gives the scene the reference builds after
  ``np.random.seed(s)``.
* :func:`synthetic_scene` builds the unit-cube fluid-block scenes used for
  throughput measurements (block of jittered particles, power-law /
  Herschel-Bulkley fluid, analytic moving cylinder rod), see :data:`CONFIGS`.
"""

import dataclasses
import math

import numpy as np

from ._abi import (DstirSceneDesc, MODEL_CARREAU, MODEL_CROSS, MODEL_HB, ROD_PARTICLES,
                   ROD_CYLINDER, J_DET, J_SVD)

# config/arguments.json of the reference (the keys the simulator reads,
# src/simulator/initialization.py:20-40)
REFERENCE_ARGUMENTS = {
    'simulation_setting': {
        'dt': 1e-3,
        'frames_per_clip': 150,
        'n_grid': 71,
        'uniform_scaling_factor': 1,
        'n_model_particles_generated': 6500,
        'n_operator_model_particles_generated': 500,
        'n_container_model_particles_generated': 500,
    },
    'scene_information': {
        'container_diameter': 0.095,
        'container_height': 0.18,
        'container_wall_thickness': 0.003,
        'liquid_height': 0.125,
        'operator_bottom_height': 0.02,
        'operator_radius': 0.0125,
        'operator_length': 0.2,
        'liquid_density': 1650,
        'operator_density': 770,
        'container_density': 1000,
    },
}

REFERENCE_BOUND = 3          # initialization.py:15
REFERENCE_BULK = 20000.0     # simulation_functions.py:112
REFERENCE_GRAVITY = -9.81    # simulation_functions.py:152
REFERENCE_CONTAINER_R = 0.0415  # simulation_functions.py:205


@dataclasses.dataclass
class Scene:
    desc: DstirSceneDesc
    liquid_x: np.ndarray           # (n_liquid, 3)
    rod_x: np.ndarray              # (n_rod, 3)
    container_x: np.ndarray        # (n_container, 3)
    trajectory: np.ndarray         # (T+1, 3), rod reference point per frame
    params: np.ndarray             # (4,)
    info: dict = dataclasses.field(default_factory=dict)

    @property
    def n_particles(self):
        return self.desc.n_liquid + self.desc.n_rod + self.desc.n_container

    def x0(self):
        return np.concatenate([self.liquid_x, self.rod_x, self.container_x], 0).astype(np.float64)

    @property
    def n_steps(self):
        return self.trajectory.shape[0] - 1


def process_trajectory(raw):
    """initialization.py:74-78: swap y and z, then centre on the bounding box."""
    t = np.asarray(raw, dtype=np.float64) @ np.array([[1, 0, 0], [0, 0, 1], [0, 1, 0]])
    centre = (np.amax(t, axis=0) - np.amin(t, axis=0)) / 2
    centre = centre + np.amin(t, axis=0)
    return t - centre, centre


def reference_like_trajectory(n_frames, dt=1e-3):
    """Analytic stand-in for the reference's data/traj.npy (before processing):
    a horizontal circle of radius 0.03 m in the file's x-y plane, starting at
    angle 0.03 rad and turning 1.889e-3 rad per 1 ms frame (2.4 turns in 8000
    frames), z = 0."""
    f = np.arange(n_frames, dtype=np.float64)
    ang = 0.029988 + 1.8891e-3 * f * (dt / 1e-3)
    return np.stack([0.03 * np.cos(ang), 0.03 * np.sin(ang), np.zeros_like(f)], 1)


def reference_constants(args=None, n_liquid=None, n_rod=None, n_container=None, n_grid=None):
    """Derived constants of initialization.py:21-54."""
    a = REFERENCE_ARGUMENTS if args is None else args
    ss, si = a['simulation_setting'], a['scene_information']
    c = {}
    c['dt'] = ss['dt']
    c['n_grid'] = n_grid if n_grid is not None else ss['n_grid']
    c['dx'] = 1 / c['n_grid']
    c['n_particles'] = n_liquid if n_liquid is not None else ss['n_model_particles_generated']
    c['n_container_particles'] = (n_container if n_container is not None
                                  else ss['n_container_model_particles_generated'])
    c['n_operator_particles'] = n_rod if n_rod is not None else ss['n_operator_model_particles_generated']
    c['uniform_scaling_factor'] = ss['uniform_scaling_factor']
    c['container_diameter'] = si['container_diameter']
    c['container_height'] = si['container_height']
    c['container_radius'] = si['container_diameter'] / 2
    c['container_wall_thickness'] = si['container_wall_thickness']
    c['liquid_height'] = si['liquid_height']
    c['operator_radius'] = si['operator_radius']
    c['operator_length'] = si['operator_length']
    c['liquid_density'] = si['liquid_density']
    c['operator_density'] = si['operator_density']
    c['container_density'] = si['container_density']
    c['operator_bottom_height'] = si['operator_bottom_height']
    c['liquid_radius'] = c['container_radius'] - c['container_wall_thickness']
    c['operator_p_vol'] = c['operator_radius'] ** 2 * c['operator_length'] * np.pi / c['n_operator_particles']
    c['liquid_p_vol'] = c['liquid_radius'] ** 2 * c['liquid_height'] * np.pi / c['n_particles']
    c['operator_p_mass'] = c['operator_density'] * c['operator_p_vol']
    c['liquid_p_mass'] = c['liquid_density'] * c['liquid_p_vol']
    area_bottom = np.pi * (c['container_radius'] ** 2)
    area_wall = c['container_diameter'] * 2 * np.pi * c['container_height']
    container_area = area_wall + area_bottom
    c['n_particles_container_wall'] = int(c['n_container_particles'] * (area_wall / container_area))
    c['n_particles_container_bottom'] = c['n_container_particles'] - c['n_particles_container_wall']
    c['container_p_vol'] = (container_area * c['container_wall_thickness']) / c['n_container_particles']
    c['container_p_mass'] = c['container_p_vol'] * c['container_density']
    return c


def sample_reference_particles(c, rod_offset, seed):
    """Rejection sampler of initialization.py:79-117 on a seeded RandomState.

    ``rod_offset`` is the reference's ``initial_pos_related_to_center``
    (initialization.py:78): the first frame of the already-centred trajectory
    minus the trajectory centre once more (see :func:`rod_offset`)."""
    rs = np.random.RandomState(seed)
    dx = c['dx']
    R, wt = c['container_radius'], c['container_wall_thickness']
    container = []
    for _ in range(c['n_particles_container_wall']):
        while True:
            x, z = rs.uniform(-R, R, 2)
            y = rs.uniform(dx + wt, dx + c['container_height'] + wt)
            if (R - wt) ** 2 <= x ** 2 + z ** 2 <= R ** 2:
                container.append((x, y, z))
                break
    for _ in range(c['n_particles_container_bottom']):
        while True:
            x, z = rs.uniform(-R, R, 2)
            y = rs.uniform(dx, dx + wt)
            if x ** 2 + z ** 2 <= R ** 2:
                container.append((x, y, z))
                break
    liquid = []
    lr = c['liquid_radius']
    for _ in range(c['n_particles']):
        while True:
            x, z = rs.uniform(-lr, lr, 2)
            y = rs.uniform(2 * dx + wt, c['liquid_height'] + wt + 2 * dx)
            if x ** 2 + z ** 2 <= lr ** 2:
                liquid.append((x, y, z))
                break
    rod = []
    orad = c['operator_radius']
    for _ in range(c['n_operator_particles']):
        while True:
            x, z = rs.uniform(-orad, orad, 2)
            y = rs.uniform(dx + c['operator_bottom_height'] + wt,
                           c['operator_length'] + c['operator_bottom_height'] + dx + wt)
            if x ** 2 + z ** 2 <= orad ** 2:
                rod.append((x, y, z))
                break
    centre = np.asarray([0.5, (REFERENCE_BOUND - 1) * dx, 0.5])
    container = np.array(container).reshape(-1, 3) + centre
    liquid = np.array(liquid).reshape(-1, 3) + centre
    rod = np.array(rod).reshape(-1, 3) + centre
    rod = rod + np.asarray(rod_offset)
    return liquid, rod, container


def rod_offset(traj_processed, centre):
    """initialization.py:78: ``operator_trajectory[0] - operator_trajectory_center``
    evaluated after the trajectory was already centred (:77), i.e. the centre
    is subtracted twice; kept as the reference computes it."""
    return np.asarray(traj_processed)[0] - np.asarray(centre)


def reference_desc(c, model=MODEL_CARREAU, j_mode=J_DET):
    d = DstirSceneDesc()
    d.n_grid = c['n_grid']
    d.bound = REFERENCE_BOUND
    d.n_liquid = c['n_particles']
    d.n_rod = c['n_operator_particles']
    d.n_container = c['n_container_particles']
    d.model = model
    d.rod_mode = ROD_PARTICLES
    d.j_mode = j_mode
    d.container_wall = 1
    d.dt = c['dt']
    d.gravity = c['uniform_scaling_factor'] * REFERENCE_GRAVITY
    d.bulk_modulus = REFERENCE_BULK
    d.liquid_p_vol = c['liquid_p_vol']
    d.liquid_p_mass = c['liquid_p_mass']
    d.rod_p_mass = c['operator_p_mass']
    d.container_p_mass = c['container_p_mass']
    d.force_scale = c['operator_p_vol'] * c['operator_density'] / c['dt']
    d.container_cx = 0.5
    d.container_cz = 0.5
    d.container_r = REFERENCE_CONTAINER_R - 0.5 * c['dx']
    d.rod_radius = 0.0
    return d


def reference_scene(seed=0, n_steps=None, raw_trajectory=None, model=MODEL_CARREAU,
                    params=(1.0, 1.0, 1.0, 1.0), n_liquid=None, n_rod=None, n_container=None,
                    n_grid=None, args=None, j_mode=J_DET):
    """The reference's stirring scene (cylindrical container, kinematic rod
    particles, 71^3 grid).  ``raw_trajectory`` is the content of
    data/traj.npy (frames x 3, before the axis swap); by default an analytic
    stand-in of 8000 frames.  ``n_steps`` truncates to the first n_steps+1
    frames (the reference uses all frames: max_steps = total_frames)."""
    if raw_trajectory is None:
        raw_trajectory = reference_like_trajectory(8000 if n_steps is None else n_steps + 1)
    raw = np.asarray(raw_trajectory, dtype=np.float64)
    if n_steps is not None:
        raw = raw[:n_steps + 1]
    c = reference_constants(args, n_liquid, n_rod, n_container, n_grid)
    traj, centre = process_trajectory(raw)
    liquid, rod, container = sample_reference_particles(c, rod_offset(traj, centre), seed)
    desc = reference_desc(c, model, j_mode)
    return Scene(desc, liquid, rod, container, traj, np.asarray(params, dtype=np.float64),
                 info={'kind': 'reference', 'seed': seed, 'constants': c})


# ---------------------------------------------------------------------------
# synthetic scenes
# ---------------------------------------------------------------------------
_PPC_SPLIT = {1: (1, 1, 1), 2: (2, 1, 1), 4: (2, 1, 2), 8: (2, 2, 2), 27: (3, 3, 3), 64: (4, 4, 4)}


def block_particles(n_grid, ppc, lo, hi, rng):
    """Jittered particles: every cell is split into ppc sub-cells (2x1x2 for 4,
    2x2x2 for 8, ...); a sub-cell whose centre lies in the box [lo, hi) holds one
    particle, placed uniformly inside that sub-cell.  Cell-major order (x, y, z
    slowest to fastest), so neighbouring particles are neighbours in space."""
    sx, sy, sz = _PPC_SPLIT[ppc]
    dx = 1.0 / n_grid
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    cl = np.floor(lo / dx).astype(int)
    ch = np.ceil(hi / dx).astype(int)
    ci = [np.arange(max(cl[d], 0), min(ch[d], n_grid)) for d in range(3)]
    cells = np.stack(np.meshgrid(*ci, indexing='ij'), -1).reshape(-1, 3)
    subs = np.stack(np.meshgrid(np.arange(sx), np.arange(sy), np.arange(sz), indexing='ij'),
                    -1).reshape(-1, 3)
    split = np.array([sx, sy, sz], float)
    centres = (cells[:, None, :] + (subs[None, :, :] + 0.5) / split) * dx
    inside = np.all((centres >= lo) & (centres < hi), axis=-1)
    corner = (cells[:, None, :] + subs[None, :, :] / split) * dx
    jit = rng.uniform(0.0, 1.0, size=centres.shape) * (dx / split)
    pos = (corner + jit)[inside]
    return pos.reshape(-1, 3)


def circle_trajectory(n_steps, dt, radius=0.15, centre=(0.5, 0.5), rev_per_s=1.0, y_tip=0.1,
                      phase=0.0):
    t = np.arange(n_steps + 1, dtype=np.float64) * dt
    ang = phase + 2 * np.pi * rev_per_s * t
    return np.stack([centre[0] + radius * np.cos(ang), np.full_like(t, y_tip),
                     centre[1] + radius * np.sin(ang)], 1)


def sinusoid_trajectory(n_steps, dt, rng, amplitude=0.2, centre=(0.5, 0.25, 0.5),
                        freq_range=(0.2, 1.5), y_tip=0.1):
    """Sum of 3 sinusoids per axis, total amplitude <= ``amplitude`` per axis
    (the y axis moves the rod tip around ``y_tip`` with a quarter of that)."""
    t = np.arange(n_steps + 1, dtype=np.float64) * dt
    out = np.zeros((n_steps + 1, 3))
    for ax in range(3):
        amp = rng.uniform(0.2, 1.0, 3)
        amp = amp / amp.sum() * (amplitude if ax != 1 else amplitude / 4)
        fr = rng.uniform(*freq_range, 3)
        ph = rng.uniform(0, 2 * np.pi, 3)
        s = sum(amp[i] * np.sin(2 * np.pi * fr[i] * t + ph[i]) for i in range(3))
        s = s - s[0]
        out[:, ax] = s
    out[:, 0] += centre[0] + 0.15
    out[:, 1] += y_tip
    out[:, 2] += centre[2]
    return out


def synthetic_desc(n_grid, ppc, n_liquid, dt=2e-4, rho=1.0, bulk=100.0, model=MODEL_HB,
                   rod_radius=0.03, j_mode=J_DET, gravity=REFERENCE_GRAVITY):
    d = DstirSceneDesc()
    d.n_grid = n_grid
    d.bound = REFERENCE_BOUND
    d.n_liquid = n_liquid
    d.n_rod = 0
    d.n_container = 0
    d.model = model
    d.rod_mode = ROD_CYLINDER
    d.j_mode = j_mode
    d.container_wall = 0
    d.dt = dt
    d.gravity = gravity
    d.bulk_modulus = bulk
    vol = (1.0 / n_grid) ** 3 / ppc
    d.liquid_p_vol = vol
    d.liquid_p_mass = rho * vol
    d.rod_p_mass = 0.0
    d.container_p_mass = 0.0
    d.force_scale = 0.0
    d.container_cx = 0.5
    d.container_cz = 0.5
    d.container_r = 1.0
    d.rod_radius = rod_radius
    return d


# Benchmark scenes.  Block extents are chosen to reach the particle counts the
# workloads are quoted at; the actual count is reported by each scene.
CONFIGS = {
    # 32^3, 4 ppc, ~14k particles, 500 substeps, K=0.5 n=0.7
    'C1': dict(n_grid=32, ppc=4, lo=(0.2, 0.05, 0.2), hi=(0.8, 0.35, 0.8), dt=2e-4, n_steps=500,
               params=(0.5, 0.0, 0.7, 0.0), rod_radius=0.03, path='circle', ckpt=50),
    # 64^3, 8 ppc, ~600k particles, 2000 substeps, checkpoint every 50
    'C2': dict(n_grid=64, ppc=8, lo=(0.1, 0.05, 0.1), hi=(0.9, 0.5, 0.9), dt=2e-4, n_steps=2000,
               params=None, rod_radius=0.03, path='circle', ckpt=50),
    # 64^3 batched, fill height U[0.15, 0.45], 1000 substeps.  n is drawn in
    # [0.4, 0.85]: draws near or above n = 1 with K ~ 1-2 exceed the explicit
    # viscous limit at dt = 2e-4 on 64^3 and blow up within ~10 substeps, in
    # the FP64 CPU restatement as on the GPU (K=1.74, n=1.04 at substep 7;
    # K=2, n=0.95 within 120 substeps; K=2, n=0.85 stays stable).
    'C3': dict(n_grid=64, ppc=8, lo=(0.2, 0.05, 0.2), hi=(0.8, None, 0.8), dt=2e-4, n_steps=1000,
               params=None, rod_radius=0.03, path='circle', ckpt=50, batch=64, yield_stress=True,
               n_range=(0.4, 0.85)),
    # 128^3, 8 ppc, ~4.8M particles, 4000 substeps, r=0.02, sinusoid path.
    # Fixed power law K=0.3, n=0.7: at dx=1/128 the explicit viscous limit of
    # dt=2e-4 is four times tighter than at 64^3, and draws such as K=1.57,
    # n=0.91 or K=0.5, n=0.9 blow up within a few hundred substeps, while
    # K=0.3, n=0.7 (and K<=2 with n<=0.5) stay stable over 1000 substeps.
    'C4': dict(n_grid=128, ppc=8, lo=(0.1, 0.05, 0.1), hi=(0.9, 0.5, 0.9), dt=2e-4, n_steps=4000,
               params=(0.3, 0.0, 0.7, 0.0), rod_radius=0.02, path='sinusoids', ckpt=100,
               k_range=(0.1, 0.5), n_range=(0.5, 0.7)),
    # 64^3, ~410k particles, 1500 substeps, identification with 16 restarts
    'C5': dict(n_grid=64, ppc=8, lo=(0.15, 0.05, 0.15), hi=(0.85, 0.45, 0.85), dt=2e-4,
               n_steps=1500, params=None, rod_radius=0.03, path='circle', ckpt=50, restarts=16,
               yield_stress=True, n_range=(0.4, 0.85)),
}


def draw_params(rng, yield_stress=False, n_range=(0.4, 1.2), k_range=(0.1, 2.0)):
    """(K, tau_y, n) of the synthetic workloads: K ~ U[k_range], n ~ U[n_range],
    tau_y ~ U[0, 5] (or 0).  Returned in the reference's parameter order
    [K, tau_y, n, unused] (simulation_functions.py:138-146)."""
    K = rng.uniform(*k_range)
    n = rng.uniform(*n_range)
    tau = rng.uniform(0.0, 5.0) if yield_stress else 0.0
    return np.array([K, tau, n, 0.0])


def config_n_range(name):
    return CONFIGS[name].get('n_range', (0.4, 1.2))


def config_k_range(name):
    return CONFIGS[name].get('k_range', (0.1, 2.0))


def draw_config_params(name, rng):
    """Seeded ground-truth parameters for configuration ``name``."""
    cfg = CONFIGS[name]
    return draw_params(rng, cfg.get('yield_stress', False), config_n_range(name), config_k_range(name))


def synthetic_scene(name='C1', seed=0, n_steps=None, n_grid=None, fill_height=None, params=None,
                    j_mode=J_DET):
    """One scene of configuration ``name`` (see :data:`CONFIGS`), seeded."""
    cfg = CONFIGS[name]
    rng = np.random.default_rng(seed)
    ng = n_grid or cfg['n_grid']
    T = n_steps if n_steps is not None else cfg['n_steps']
    lo = list(cfg['lo'])
    hi = list(cfg['hi'])
    if hi[1] is None:
        hi[1] = fill_height if fill_height is not None else rng.uniform(0.15, 0.45)
    pos = block_particles(ng, cfg['ppc'], lo, hi, rng)
    if params is None:
        params = cfg['params'] if cfg['params'] is not None else draw_config_params(name, rng)
    if cfg['path'] == 'circle':
        traj = circle_trajectory(T, cfg['dt'])
    else:
        traj = sinusoid_trajectory(T, cfg['dt'], rng)
    desc = synthetic_desc(ng, cfg['ppc'], pos.shape[0], dt=cfg['dt'], rod_radius=cfg['rod_radius'],
                          j_mode=j_mode)
    z = np.zeros((0, 3))
    return Scene(desc, pos, z, z, traj, np.asarray(params, dtype=np.float64),
                 info={'kind': 'synthetic', 'config': name, 'seed': seed, 'fill_top': hi[1]})


def small_synthetic_scene(n_grid=16, ppc=1, n_steps=10, seed=0, lo=(0.3, 0.12, 0.3),
                          hi=(0.7, 0.4, 0.7), params=(0.5, 0.0, 0.7, 0.0), model=MODEL_HB,
                          dt=2e-4, rod_radius=0.06, j_mode=J_DET, bulk=100.0):
    """A small cylinder-rod scene for parity tests (oracle-sized)."""
    rng = np.random.default_rng(seed)
    pos = block_particles(n_grid, ppc, lo, hi, rng)
    traj = circle_trajectory(n_steps, dt, radius=0.08, y_tip=0.15)
    desc = synthetic_desc(n_grid, ppc, pos.shape[0], dt=dt, rod_radius=rod_radius, model=model,
                          j_mode=j_mode, bulk=bulk)
    z = np.zeros((0, 3))
    return Scene(desc, pos, z, z, traj, np.asarray(params, dtype=np.float64),
                 info={'kind': 'synthetic-small', 'seed': seed})


__all__ = ['Scene', 'reference_scene', 'synthetic_scene', 'small_synthetic_scene', 'CONFIGS',
           'process_trajectory', 'reference_like_trajectory', 'reference_constants',
           'reference_desc', 'block_particles', 'circle_trajectory', 'sinusoid_trajectory',
           'MODEL_CARREAU', 'MODEL_CROSS', 'MODEL_HB', 'ROD_PARTICLES', 'ROD_CYLINDER',
           'J_DET', 'J_SVD']
