"""Helpers that turn a golden fixture (tests/golden/*.npz) into oracle / GPU inputs."""

import os

import numpy as np

from diffstir_gb300._abi import DstirSceneDesc, ROD_PARTICLES, J_DET

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def load(name):
    return np.load(os.path.join(GOLDEN_DIR, name + '.npz'))


def desc_from_fixture(d, model):
    g = lambda k: float(d['scene_' + k])
    desc = DstirSceneDesc()
    desc.n_grid = int(g('n_grid'))
    desc.bound = int(g('bound'))
    desc.n_liquid = int(g('n_particles'))
    desc.n_rod = int(g('n_operator_particles'))
    desc.n_container = int(g('n_container_particles'))
    desc.model = model
    desc.rod_mode = ROD_PARTICLES
    desc.j_mode = J_DET
    desc.container_wall = 1
    desc.dt = g('dt')
    desc.gravity = -9.81 * g('uniform_scaling_factor')
    desc.bulk_modulus = 20000.0
    desc.liquid_p_vol = g('liquid_p_vol')
    desc.liquid_p_mass = g('liquid_p_mass')
    desc.rod_p_mass = g('operator_p_mass')
    desc.container_p_mass = g('container_p_mass')
    desc.force_scale = g('operator_p_vol') * g('operator_density') / g('dt')
    desc.container_cx = 0.5
    desc.container_cz = 0.5
    desc.container_r = 0.0415 - 0.5 * g('dx')
    desc.rod_radius = 0.0
    return desc


def inputs(d):
    x0 = np.concatenate([d['liquid_particles'], d['operator_particles'], d['container_particles']], 0)
    traj = d['operator_trajectory']
    T = traj.shape[0] - 1
    return x0, traj, T


def reference_loss_and_dforce(force, target, T):
    """compute_loss (simulation_functions.py:330-339) on a force profile whose
    entry f is the reference's frame f+1; returns (loss, dL/dforce [T,3])."""
    fx = np.concatenate([[0.0], force[:T - 1, 0]])          # frames 0..T-1
    diff = fx - target[:T]
    loss = np.abs(diff).sum() / T
    dF = np.zeros((T, 3))
    dF[:T - 1, 0] = np.sign(diff[1:]) / T
    return loss, dF
