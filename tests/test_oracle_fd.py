"""Central finite differences of the FP64 oracle (its adjoint is exact for the
restated equations), on the parts of the path the reference scene does not
exercise: the moving-cylinder rod, the SVD-determinant mode, the three models
with the MSE force loss of the synthetic scenes, and the SVD kernels."""

import os

import numpy as np
import pytest

import oracle
from diffstir_gb300 import scene as S


def _loss_and_grad(sc, T, wts, params=None, want_state0=False, x0=None):
    p = sc.params if params is None else params
    x = sc.x0() if x0 is None else x0
    force, _, _ = oracle.rollout(sc.desc, p, sc.trajectory, T, x)
    loss = float((wts * force).sum())
    _, dp, ds, _ = oracle.grad(sc.desc, p, sc.trajectory, T, x, wts, want_state0=want_state0)
    return loss, dp, ds


def _fd_params(sc, T, wts, idx, h_rel=1e-6):
    out = []
    for i in idx:
        p = sc.params.copy()
        h = h_rel * max(abs(p[i]), 1e-3)
        p[i] += h
        fp, _, _ = oracle.rollout(sc.desc, p, sc.trajectory, T, sc.x0())
        p[i] -= 2 * h
        fm, _, _ = oracle.rollout(sc.desc, p, sc.trajectory, T, sc.x0())
        out.append(float((wts * (fp - fm)).sum()) / (2 * h))
    return np.array(out)


MODELS = [
    (S.MODEL_HB, (0.5, 0.3, 0.7, 0.0), (0, 1, 2)),
    (S.MODEL_CARREAU, (2.0, 0.1, 0.6, 0.8), (0, 1, 2, 3)),
    (S.MODEL_CROSS, (1.5, 0.2, 0.5, 1.2), (0, 1, 2, 3)),
]


@pytest.mark.parametrize('model,params,idx', MODELS)
@pytest.mark.parametrize('j_mode', [S.J_DET, S.J_SVD])
def test_cylinder_scene_param_grad_fd(model, params, idx, j_mode):
    T = 12
    sc = S.small_synthetic_scene(n_grid=12, ppc=2, n_steps=T, params=params, model=model, j_mode=j_mode,
                                 seed=3, dt=5e-4)
    rng = np.random.default_rng(7)
    wts = rng.normal(size=(T, 3))
    loss, dp, _ = _loss_and_grad(sc, T, wts)
    fd = _fd_params(sc, T, wts, idx)
    assert np.any(np.abs(fd) > 0)
    np.testing.assert_allclose(dp[list(idx)], fd, rtol=2e-5, atol=1e-9 * np.abs(fd).max())


def test_cylinder_scene_state_grad_fd():
    T = 10
    sc = S.small_synthetic_scene(n_grid=12, ppc=2, n_steps=T, seed=5, dt=5e-4)
    rng = np.random.default_rng(1)
    wts = rng.normal(size=(T, 3))
    _, _, ds = _loss_and_grad(sc, T, wts, want_state0=True)
    x0 = sc.x0()
    for p in rng.choice(x0.shape[0], 4, replace=False):
        for c in range(3):
            h = 1e-7
            xp, xm = x0.copy(), x0.copy()
            xp[p, c] += h
            xm[p, c] -= h
            fp, _, _ = oracle.rollout(sc.desc, sc.params, sc.trajectory, T, xp)
            fm, _, _ = oracle.rollout(sc.desc, sc.params, sc.trajectory, T, xm)
            fd = float((wts * (fp - fm)).sum()) / (2 * h)
            assert abs(ds[p, c] - fd) <= 1e-4 * max(abs(fd), np.abs(ds[:, :3]).max() * 1e-2), (p, c, ds[p, c], fd)


@pytest.mark.parametrize('j_mode', [S.J_DET, S.J_SVD])
def test_state_adjoint_dot_product(j_mode):
    """Dot-product test of the whole reverse pass on the FP64 oracle: for a
    random direction u over all 24 components (x, v, C, F) of every
    particle's step-0 state, <w, J u> by central differences of the forces
    along u equals <J^T w, u> from the adjoint of the step-0 state."""
    T = 10
    sc = S.small_synthetic_scene(n_grid=12, ppc=2, n_steps=T, seed=8, dt=5e-4, j_mode=j_mode)
    rng = np.random.default_rng(11)
    wts = rng.normal(size=(T, 3))
    x0 = sc.x0()
    n = x0.shape[0]
    v0 = rng.normal(scale=0.05, size=(n, 3))
    C0 = rng.normal(scale=0.2, size=(n, 9))
    F0 = np.tile(np.eye(3).reshape(1, 9), (n, 1)) + rng.normal(scale=0.01, size=(n, 9))
    _, _, ds, st = oracle.grad(sc.desc, sc.params, sc.trajectory, T, x0, wts, v0, C0, F0, want_state0=True)
    assert st == 0
    u = rng.normal(size=(n, 24))
    u[:, :3] *= 1e-2  # positions: keep the perturbed stencils comparable to the others
    h = 1e-6

    def proj(sign):
        f, _, _ = oracle.rollout(sc.desc, sc.params, sc.trajectory, T, x0 + sign * h * u[:, :3],
                                 v0 + sign * h * u[:, 3:6], C0 + sign * h * u[:, 6:15], F0 + sign * h * u[:, 15:])
        return float((wts * f).sum())

    jvp = (proj(1) - proj(-1)) / (2 * h)
    vjp = float((ds * u).sum())
    assert abs(jvp) > 0
    assert abs(vjp - jvp) <= 1e-6 * abs(jvp), (vjp, jvp)


def test_reference_scene_param_grad_fd():
    """Reference scene (container, rod particles, k=20000), L1 loss as compute_loss."""
    T = 6
    sc = S.reference_scene(seed=0, n_steps=T, n_liquid=300, n_rod=40, n_container=60, n_grid=32,
                           model=S.MODEL_CARREAU, params=(2.0, 0.1, 0.6, 0.8))
    rng = np.random.default_rng(2)
    wts = rng.normal(size=(T, 3))
    _, dp, _ = _loss_and_grad(sc, T, wts)
    fd = _fd_params(sc, T, wts, (0, 1, 2, 3))
    np.testing.assert_allclose(dp, fd, rtol=2e-4, atol=1e-6 * np.abs(fd).max())


def test_svd3_matches_numpy():
    rng = np.random.default_rng(0)
    A = rng.normal(size=(200, 3, 3))
    A[:50] = np.eye(3) + 0.05 * rng.normal(size=(50, 3, 3))
    A[50:60] = np.diag([1.0, 1.0, 1.0]) + 1e-7 * rng.normal(size=(10, 3, 3))
    U, Sg, V = oracle.svd3(A)
    rec = np.einsum('nij,nj,nkj->nik', U, Sg, V)
    np.testing.assert_allclose(rec, A, atol=1e-10)
    eye = np.broadcast_to(np.eye(3), U.shape)
    np.testing.assert_allclose(np.einsum('nji,njk->nik', U, U), eye, atol=1e-10)
    np.testing.assert_allclose(np.einsum('nji,njk->nik', V, V), eye, atol=1e-10)
    assert np.all(np.linalg.det(U) > 0) and np.all(np.linalg.det(V) > 0)
    ref = np.linalg.svd(A, compute_uv=False)
    np.testing.assert_allclose(np.abs(Sg), ref, rtol=1e-9, atol=1e-12)
    assert np.all(Sg[:, 0] >= Sg[:, 1]) and np.all(Sg[:, 1] >= np.abs(Sg[:, 2]) - 1e-12)
    np.testing.assert_allclose(np.sign(Sg[:, 2]), np.sign(np.linalg.det(A)))


def test_svd3_backward_fd():
    rng = np.random.default_rng(1)
    A = rng.normal(size=(20, 3, 3))
    gU, gS, gV = rng.normal(size=(20, 3, 3)), rng.normal(size=(20, 3)), rng.normal(size=(20, 3, 3))
    U, Sg, V = oracle.svd3(A)
    gA = oracle.svd3_backward(gU, gS, gV, U, Sg, V)
    h = 1e-6
    for n in range(5):
        for i in range(3):
            for j in range(3):
                Ap, Am = A[n:n + 1].copy(), A[n:n + 1].copy()
                Ap[0, i, j] += h
                Am[0, i, j] -= h
                Up, Sp, Vp = oracle.svd3(Ap)
                Um, Sm, Vm = oracle.svd3(Am)
                L = lambda u, s, v: (gU[n] * u[0]).sum() + (gS[n] * s[0]).sum() + (gV[n] * v[0]).sum()
                fd = (L(Up, Sp, Vp) - L(Um, Sm, Vm)) / (2 * h)
                assert abs(gA[n, i, j] - fd) < 1e-5 * max(1.0, abs(fd)), (n, i, j, gA[n, i, j], fd)


def test_segment_chaining_equals_one_shot():
    """The segment forms (rollout returning the last state, reverse pass
    seeded with the adjoint of the final state) chained over four segments
    reproduce the one-shot FP64 rollout and gradient."""
    T, K = 40, 10
    sc = S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=3)
    w = np.random.default_rng(0).normal(size=(T, 3))
    f1, dp1, ds1, _ = oracle.grad(sc.desc, sc.params, sc.trajectory, T, sc.x0(), w, want_state0=True)
    state = (sc.x0(), None, None, None)
    ckpts, forces = [], []
    for s0 in range(0, T, K):
        ckpts.append(state)
        f, last, st = oracle.rollout_last(sc.desc, sc.params, sc.trajectory[s0:s0 + K + 1], K, *state)
        assert st == 0
        forces.append(f)
        state = (last[:, 0:3], last[:, 3:6], last[:, 6:15], last[:, 15:24])
    np.testing.assert_allclose(np.concatenate(forces), f1, rtol=0, atol=1e-12 * np.abs(f1).max())
    adj, dp = None, np.zeros(4)
    for i in reversed(range(len(ckpts))):
        s0 = i * K
        x, v, C, F = ckpts[i]
        _, d, adj, _ = oracle.grad_seeded(sc.desc, sc.params, sc.trajectory[s0:s0 + K + 1], K, x, w[s0:s0 + K], adj,
                                          v, C, F)
        dp += d
    np.testing.assert_allclose(dp, dp1, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(adj, ds1, rtol=1e-12, atol=1e-14)


@pytest.mark.skipif(not os.environ.get('DIFFSTIR_SLOW'), reason='several minutes of CPU; set DIFFSTIR_SLOW=1')
def test_sticky_top_is_what_separates_adjoint_and_differences():
    """The 64^3 workload's block and parameters at 32^3 over 1000 substeps: the
    fluid reaches the top band (j > n - bound) after ~300 substeps.  With the
    reference's sticky top (a top-band node loses its whole velocity when
    v_y > 0, simulation_functions.py:221-224) the loss has many small jumps in
    the parameters, so central differences (h = 1e-4 x |param|) move away from
    the adjoint; with that rule replaced by a plain clamp of v_y the two agree
    to 1e-5 again.  FP64 throughout."""
    cfg = S.CONFIGS['C2']
    p = np.array([0.11404720693826675, 0.0, 0.8690828084945679, 0.0])
    truth = S.draw_config_params('C2', np.random.default_rng(1000))
    pos = S.block_particles(32, 8, cfg['lo'], cfg['hi'], np.random.default_rng(0))
    desc = S.synthetic_desc(32, 8, pos.shape[0], dt=cfg['dt'], rod_radius=cfg['rod_radius'])
    T = 1000
    traj = S.circle_trajectory(T, cfg['dt'])
    thr = oracle.max_threads()
    gaps = {}
    for variant in (None, 'continuous_top'):
        ft, _, st = oracle.rollout(desc, truth, traj, T, pos, threads=thr, variant=variant)
        assert st == 0

        def loss(pp):
            f, _, s = oracle.rollout(desc, pp, traj, T, pos, threads=thr, variant=variant)
            d = (f - ft)[:, 0::2]
            return (d * d).sum() / d.size, f

        _, f0 = loss(p)
        d = (f0 - ft)[:, 0::2]
        w = np.zeros((T, 3))
        w[:, 0::2] = 2 * d / d.size
        _, dp, _, _ = oracle.grad(desc, p, traj, T, pos, w, threads=thr, variant=variant)
        rel = []
        for i in (0, 2):
            h = 1e-4 * abs(p[i])
            pp, pm = p.copy(), p.copy()
            pp[i] += h
            pm[i] -= h
            fd = (loss(pp)[0] - loss(pm)[0]) / (2 * h)
            rel.append(abs(fd - dp[i]) / abs(fd))
        gaps[variant] = max(rel)
    assert gaps[None] > 1e-3
    assert gaps['continuous_top'] < 1e-5


@pytest.mark.parametrize('T', [1, 3])
def test_state_to_state_adjoint_dot_product(T):
    """Dot-product test of the state-to-state adjoint of whole substeps (P2G,
    grid update and G2P with their adjoints): with a random adjoint W of the
    final state and random weights w of the forces, <W, dS_T/dS_0 u> +
    <w, dF/dS_0 u> by central differences along a random full-state
    direction u equals <dL/dS_0, u> from the reverse pass seeded with W."""
    sc = S.small_synthetic_scene(n_grid=12, ppc=2, n_steps=T, seed=9, dt=5e-4)
    rng = np.random.default_rng(17)
    x0 = sc.x0()
    n = x0.shape[0]
    v0 = rng.normal(scale=0.05, size=(n, 3))
    C0 = rng.normal(scale=0.2, size=(n, 9))
    F0 = np.tile(np.eye(3).reshape(1, 9), (n, 1)) + rng.normal(scale=0.01, size=(n, 9))
    wts = rng.normal(size=(T, 3))
    W = rng.normal(size=(n, 24))
    _, _, ds, st = oracle.grad_seeded(sc.desc, sc.params, sc.trajectory, T, x0, wts, W, v0, C0, F0)
    assert st == 0
    u = rng.normal(size=(n, 24))
    u[:, :3] *= 1e-2
    h = 1e-6

    def proj(sign):
        f, last, _ = oracle.rollout_last(sc.desc, sc.params, sc.trajectory, T, x0 + sign * h * u[:, :3],
                                         v0 + sign * h * u[:, 3:6], C0 + sign * h * u[:, 6:15],
                                         F0 + sign * h * u[:, 15:])
        return float((wts * f).sum()) + float((W * last).sum())

    jvp = (proj(1) - proj(-1)) / (2 * h)
    vjp = float((ds * u).sum())
    assert abs(jvp) > 0
    assert abs(vjp - jvp) <= 1e-6 * abs(jvp), (vjp, jvp)
