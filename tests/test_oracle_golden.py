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

FIXTURES = [('ref_f64_g32', 'f64', (0, 1, 2)), ('ref_f32_g32', 'f32', (0, 1, 2)), ('ref_f64_g71', 'f64', (2,))]
CASES = [(n, p, m) for (n, p, ms) in FIXTURES for m in ms]

# relative tolerances: (force, state, param grad, state grad)
TOL = {'f64': (2e-6, 2e-6, 2e-6, 2e-6), 'f32': (2e-3, 2e-4, 2e-2, 2e-2)}


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
    tf, ts, tg, tsg = TOL[prec]
    # states of every step: liquid x, v, C, F; rod C; container C
    assert _rel(states[:, :nl, 0:3], d[p + 'x']) < ts
    assert _rel(states[:, :nl, 3:6], d[p + 'v']) < max(ts, 1e-5)
    assert _rel(states[:, :nl, 6:15].reshape(T + 1, nl, 3, 3), d[p + 'C']) < ts * 10
    assert _rel(states[:, :nl, 15:24].reshape(T + 1, nl, 3, 3), d[p + 'F']) < ts
    nr = desc.n_rod
    assert _rel(states[:, nl:nl + nr, 6:15].reshape(T + 1, nr, 3, 3), d[p + 'operator_C']) < ts * 10
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
