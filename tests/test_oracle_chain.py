"""The segment-chained FP64 oracle (oracle.rollout_chain) used for long
horizons of large scenes: chaining K-substep segments, and seeding each
segment's reverse pass with the later segment's state adjoint, reproduces the
one-call rollout and gradient."""

import numpy as np

import oracle
from diffstir_gb300 import scene as S


def test_chained_rollout_and_gradient_equal_one_call():
    T = 13
    sc = S.small_synthetic_scene(n_grid=12, ppc=2, n_steps=T, seed=5, params=(0.9, 0.3, 0.7, 0.0))
    w = np.random.default_rng(2).normal(size=(T, 3))
    f1, _, _ = oracle.rollout(sc.desc, sc.params, sc.trajectory, T, sc.x0())
    _, dp1, _, _ = oracle.grad(sc.desc, sc.params, sc.trajectory, T, sc.x0(), w)
    f2 = oracle.rollout_chain(sc.desc, sc.params, sc.trajectory, T, sc.x0(), 5)
    f3, dp3 = oracle.rollout_chain(sc.desc, sc.params, sc.trajectory, T, sc.x0(), 5, w=w)
    np.testing.assert_allclose(f2, f1, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(f3, f1, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(dp3, dp1, rtol=1e-10, atol=1e-14 * np.abs(dp1).max())
