"""Host-side logic without a GPU: the reference-scene builder against the
scene the reference's own code built (golden fixtures), the compat module's
API surface, the reference's step rule, the synthetic scene generators, and the launch
options the autotuner and the bench pass against the header's list."""

import os

import numpy as np
import pytest

import golden_util as gu
from diffstir_gb300 import scene as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize('name', ['ref_f64_g32', 'ref_f64_g71'])
def test_reference_scene_sampler_matches_reference_source(name):
    d = gu.load(name)
    seed = int(d['meta_seed'])
    n_grid = int(d['scene_n_grid'])
    nl, nr, nc = (int(d['scene_n_particles']), int(d['scene_n_operator_particles']),
                  int(d['scene_n_container_particles']))
    c = S.reference_constants(None, nl, nr, nc, n_grid)
    for k in ('liquid_p_vol', 'liquid_p_mass', 'operator_p_vol', 'operator_p_mass', 'container_p_vol',
              'container_p_mass', 'n_particles_container_wall', 'n_particles_container_bottom', 'dx'):
        assert np.isclose(c[k], float(d['scene_' + k]), rtol=1e-15, atol=0), k
    if 'raw_trajectory' not in d.files:
        pytest.skip('fixture predates the raw trajectory record')
    t, centre = S.process_trajectory(d['raw_trajectory'])
    np.testing.assert_allclose(t, d['operator_trajectory'], rtol=0, atol=1e-15)
    liquid, rod, cont = S.sample_reference_particles(c, S.rod_offset(t, centre), seed)
    np.testing.assert_array_equal(liquid, d['liquid_particles'])
    np.testing.assert_array_equal(rod, d['operator_particles'])
    np.testing.assert_array_equal(cont, d['container_particles'])


def test_reference_desc_constants():
    c = S.reference_constants()
    d = S.reference_desc(c)
    assert d.n_grid == 71 and d.bound == 3 and d.n_liquid == 6500 and d.n_rod == 500 and d.n_container == 500
    assert np.isclose(d.container_r, 0.0415 - 0.5 / 71)
    assert np.isclose(d.force_scale, c['operator_p_vol'] * 770 / 1e-3, rtol=1e-6)
    assert np.isclose(d.bulk_modulus, 20000.0)


def test_reference_like_trajectory_shape_and_rate():
    raw = S.reference_like_trajectory(8000)
    assert raw.shape == (8000, 3)
    r = np.hypot(raw[:, 0], raw[:, 1])
    assert np.allclose(r, 0.03)
    turns = (np.unwrap(np.arctan2(raw[:, 1], raw[:, 0]))[-1] - np.arctan2(raw[0, 1], raw[0, 0])) / (2 * np.pi)
    assert 2.35 < turns < 2.45


def test_synthetic_scene_counts():
    sc = S.synthetic_scene('C1', seed=0, n_steps=10)
    assert 12500 < sc.n_particles < 15000
    x = sc.x0()
    assert x[:, 0].min() >= 0.2 and x[:, 0].max() <= 0.8 and x[:, 1].min() >= 0.05 and x[:, 1].max() <= 0.35
    sc2 = S.synthetic_scene('C2', seed=0, n_steps=4)
    assert 590000 < sc2.n_particles < 620000
    t = S.synthetic_scene('C4', seed=3, n_steps=50).trajectory
    assert np.abs(t[:, 0] - t[0, 0]).max() <= 0.4 + 1e-9
    a = S.synthetic_scene('C3', seed=1, n_steps=4)
    b = S.synthetic_scene('C3', seed=2, n_steps=4)
    assert a.n_particles != b.n_particles


def test_compat_exposes_reference_names():
    from diffstir_gb300 import compat as sf
    names = ['initialize_objects', 'initialize_ti_field', 'forward', 'backward', 'compute_loss', 'ti', 'loss',
             'model_index', 'constitutive_parameters', 'learning_rate', 'parameters_lower_bound',
             'parameters_upper_bound', 'x', 'operator_x', 'container_x', 'initial_x', 'initial_operator_x',
             'operator_kinematic_seq', 'operator_forces_seq', 'total_operator_dv', 'max_steps', 'dt', 'dx',
             'inv_dx', 'n_grid', 'bound', 'n_clips', 'frames_per_clip', 'operator_p_vol', 'operator_density',
             'n_constitutive_parameters', 'operator_trajectory', 'force_magnitudes', 'liquid_p_mass']
    for n in names:
        assert hasattr(sf, n), n
    assert sf.max_steps == 8000 and sf.n_clips == 53 and sf.frames_per_clip == 150
    assert hasattr(sf.ti.ad, 'Tape') and hasattr(sf.constitutive_parameters, 'grad')
    sf.constitutive_parameters[2] = 0.5
    assert sf.constitutive_parameters[2] == pytest.approx(0.5)
    sf.model_index[None] = 2
    assert sf.model_index[None] == 2


def test_single_parameter_fitting1_rule():
    from diffstir_gb300 import identify
    assert identify.magnitude_level(0.0) == -11 and identify.magnitude_level(123.0) == 2
    p, lr = identify.single_parameter_fitting1(1.0, 0.5, 0.0, 10.0, 1.0, 35, 0)
    assert 0.0 < p < 10.0 and lr > 0
    assert identify.single_parameter_fitting1(1.0, 0.0, 0.0, 10.0, 1.0, 35, 3) == (1.0, 1.0)
    # coinciding bounds (the reference config's all-ones case) terminates
    p3, _ = identify.single_parameter_fitting1(1.0, 0.3, 1.0, 1.0, 1.0, 35, 2)
    assert np.isfinite(p3)


def test_product_fails_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    from diffstir_gb300.simulator import Simulator
    with pytest.raises(RuntimeError):
        Simulator(S.small_synthetic_scene(n_steps=2))


def _documented_options():
    import re
    src = open(os.path.join(ROOT, 'include', 'diffstir.h')).read()
    i, j = src.index('/* Tuning knobs'), src.index('int dstir_set_option')
    return set(re.findall(r'"([a-z_0-9]+)"', src[i:j]))


def test_autotune_candidates_use_documented_options():
    from diffstir_gb300 import autotune
    keys = _documented_options()
    for cand in autotune.CANDIDATES:
        assert set(cand) <= keys, set(cand) - keys


def test_bench_option_flags_are_documented_options():
    import re
    src = open(os.path.join(ROOT, 'bench.py')).read()
    m = re.search(r"keys = \(([^)]*)\)", src)
    names = set(re.findall(r"'([a-z_0-9]+)'", m.group(1)))
    assert names and names <= _documented_options(), names - _documented_options()


def test_prefetch_hint_addresses_stay_in_the_block():
    """Host restatement of prefetch_state_l2 (device_util.cuh): for blocks of
    up to 256 particles at any start offset, every address that threads
    0..255 touch lies inside the block's particle range, and the 128-byte
    lines they touch are exactly the lines that hold the block's particles,
    for every requested component."""
    rng = np.random.default_rng(3)
    for _ in range(200):
        start = int(rng.integers(0, 10**6))
        count = int(rng.integers(1, 257))
        end = start + count
        ncomp = int(rng.integers(1, 25))
        stride = 10**6 + 512                          # a multiple of 32, as the handle's stride
        touched = {}
        for t in range(256):
            comp, line = divmod(t, 9)
            if comp >= ncomp:
                continue
            p = min(start + 32 * line, end - 1)
            assert start <= p < end
            touched.setdefault(comp, []).append(comp * stride + p)
        assert sorted(touched) == list(range(ncomp))
        for comp, addrs in touched.items():
            base = comp * stride                         # a 128-byte-aligned base: stride % 32 == 0
            lines = {a // 32 for a in addrs}             # float index -> 128-byte line
            assert lines == {(base + q) // 32 for q in range(start, end)}
