"""Oracle (oracle/oracle.cpp) against golden fixtures produced by executing the
reference's own simulator source (tests/golden/make_golden.py).

The f64 fixtures pin the algorithm: the reference's forward(s)/compute_loss and
its Taichi-semantics reverse mode, evaluated in float64, agree with the FP64
oracle to the float32 rounding of the scene constants (DstirSceneDesc stores
them as float).  The f32 fixtures compare the FP32 build with the reference's
every-operation-rounded float32 evaluation.
"""

import os

import numpy as np
import pytest

import golden_util as gu
import oracle

FIXTURES = [('ref_f64_g32', 'f64', (0, 1, 2)), ('ref_f32_g32', 'f32', (0, 1, 2)), ('ref_f64_g71', 'f64', (2,)),
            ('ref_f64_g16_long', 'f64', (0, 1, 2)), ('ref_f32_g16_long', 'f32', (0, 1, 2))]
CASES = [(n, p, m) for (n, p, ms) in FIXTURES for m in ms]

# relative tolerances: (force, state, param grad, state grad).  Measured
# worst cases over all fixtures and models: f64 1.2e-7 (state), f32 2.0e-6
# (force and state) and 1.3e-6 (gradients); the bars leave a factor of ten.
TOL = {'f64': (2e-6, 2e-6, 2e-6, 2e-6), 'f32': (2e-5, 2e-5, 2e-5, 2e-5)}


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.mark.parametrize('name,prec,model', CASES)
def test_oracle_matches_reference_source(name, prec, model):
    path = os.path.join(gu.GOLDEN_DIR, name + '.npz')
    if not os.path.exists(path):
        pytest.skip('fixture %s not generated' % name)
    d = np.load(path)
    p = 'm%d_' % model
    desc = gu.desc_from_fixture(d, model)
    x0, traj, T = gu.inputs(d)
    nl = desc.n_liquid
    force, states, status = oracle.rollout(desc, d[p + 'params'], traj, T, x0, precision=prec,
                                           return_states=True)
    assert status == 0
    # long fixtures keep every stride-th frame's particle state only
    stride = int(d['meta_state_stride']) if 'meta_state_stride' in d.files else 1
    states = states[::stride]
    nf = states.shape[0]
    tf, ts, tg, tsg = TOL[prec]
    # states of every (stored) step: liquid x, v, C, F; rod C; container C
    assert _rel(states[:, :nl, 0:3], d[p + 'x']) < ts
    assert _rel(states[:, :nl, 3:6], d[p + 'v']) < max(ts, 1e-5)
    assert _rel(states[:, :nl, 6:15].reshape(nf, nl, 3, 3), d[p + 'C']) < ts * 10
    assert _rel(states[:, :nl, 15:24].reshape(nf, nl, 3, 3), d[p + 'F']) < ts
    nr = desc.n_rod
    assert _rel(states[:, nl:nl + nr, 6:15].reshape(nf, nr, 3, 3), d[p + 'operator_C']) < ts * 10
    # reaction force: reference total_operator_dv[f+1] * V_o rho_o / dt
    ref_force = d[p + 'total_operator_dv'] * desc.force_scale
    assert _rel(force[:T - 1], ref_force[1:T]) < tf
    loss, dF = gu.reference_loss_and_dforce(force, d[p + 'target'], T)
    assert abs(loss - float(d[p + 'loss'])) <= tf * abs(float(d[p + 'loss']))
    if p + 'grad_params' not in d.files:
        return
    _, dp, ds, _ = oracle.grad(desc, d[p + 'params'], traj, T, x0, dF, precision=prec, want_state0=True)
    gp = d[p + 'grad_params']
    assert _rel(dp, gp) < tg, (dp, gp)
    assert _rel(ds[:nl, 0:3], d[p + 'grad_x0']) < tsg
    assert _rel(ds[:nl, 3:6], d[p + 'grad_v0']) < tsg
    assert _rel(ds[:nl, 15:24], d[p + 'grad_F0'].reshape(nl, 9)) < tsg


def test_long_fixtures_reach_every_boundary_rule():
    """The long fixtures' rollouts (60 substeps of the reference's own code)
    exercise every boundary rule of grid_op on nodes with mass: the container
    projection (simulation_functions.py:205-210), the six wall clamps
    (:211-220) and the sticky top (:221-224), counted by the oracle's
    branch-count build over the same rollout."""
    for name in ('ref_f64_g16_long', 'ref_f32_g16_long'):
        path = os.path.join(gu.GOLDEN_DIR, name + '.npz')
        if not os.path.exists(path):
            pytest.skip('fixture %s not generated' % name)
        d = np.load(path)
        x0, traj, T = gu.inputs(d)
        assert T >= 50
        # the rod velocity (q[f+1]-q[f])/dt needs no float32 rounding of q
        assert np.array_equal(traj.astype(np.float32).astype(np.float64), traj)
        for model in (0, 1, 2):
            oracle.branch_counts()
            oracle.rollout(gu.desc_from_fixture(d, model), d['m%d_params' % model], traj, T, x0,
                           variant='branch_counts')
            counts = oracle.branch_counts()
            for rule in oracle.BRANCHES:
                assert counts[rule] > 100, (name, model, rule, counts)
            # and the rod dv accumulates a nonzero reaction force in every frame compute_loss sums
            assert np.all(np.abs(d['m%d_total_operator_dv' % model][1:T]).sum(axis=1) > 0)
