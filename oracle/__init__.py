"""CPU oracle of the DiffStir MLS-MPM path (test infrastructure).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm may import this package, and only as the checker or as the timed CPU
stand-in for the reference; the diffstir_gb300 product never does.

``build()`` compiles oracle.cpp (a line-by-line C++ restatement of
src/simulator/simulation_functions.py with a hand-derived adjoint) into
``oracle/_build/liboracle.so`` with g++ and OpenMP.  The diagnostic variant
``continuous_top`` (``liboracle_continuous_top.so``) replaces the reference's
sticky top (a node of the top band loses its whole velocity when v_y > 0,
simulation_functions.py:221-224) by a clamp of v_y alone; it exists only to
show that this discontinuous rule is what separates adjoint and difference
quotients once the fluid reaches the top band.  The diagnostic variant
``branch_counts`` counts how often each boundary rule of grid_op
(simulation_functions.py:204-224) changed the velocity of a node with mass
(:func:`branch_counts`), to show which rules a fixture's rollout exercises.
"""

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'oracle.cpp')
OUT_DIR = os.path.join(HERE, '_build')
LIB = os.path.join(OUT_DIR, 'liboracle.so')
VARIANTS = {None: ([], 'liboracle.so'),
            'continuous_top': (['-DORACLE_CONTINUOUS_TOP'], 'liboracle_continuous_top.so'),
            'branch_counts': (['-DORACLE_BRANCH_COUNTS'], 'liboracle_branch_counts.so')}
BRANCHES = ('container_projection', 'wall_i_low', 'wall_i_high', 'wall_k_low', 'wall_k_high', 'wall_j_low',
            'sticky_top', 'nodes_with_mass')

_libs = {}


def build(force=False, variant=None):
    os.makedirs(OUT_DIR, exist_ok=True)
    flags, name = VARIANTS[variant]
    lib = os.path.join(OUT_DIR, name)
    hdr = os.path.join(HERE, '..', 'include', 'diffstir.h')
    if (not force and os.path.exists(lib)
            and os.path.getmtime(lib) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr),
                                             os.path.getmtime(__file__))):
        return lib
    tmp = lib + '.tmp%d' % os.getpid()
    # -ffp-contract=off: every operation rounded as written (no fused
    # multiply-adds), so that the FP32 build follows the reference's
    # per-operation rounding and gives the same results on x86-64 and aarch64
    cmd = ['g++', '-O2', '-std=c++17', '-ffp-contract=off', '-fopenmp', '-fPIC', '-shared'] + flags + ['-o', tmp, SRC]
    subprocess.run(cmd, check=True)
    os.replace(tmp, lib)
    return lib


def load(variant=None):
    if variant not in _libs:
        from diffstir_gb300._abi import DstirSceneDesc
        lib = C.CDLL(build(variant=variant))
        D = C.POINTER(C.c_double)
        sig_roll = [C.POINTER(DstirSceneDesc), D, D, C.c_int, D, D, D, D, D, D, C.c_int]
        sig_grad = [C.POINTER(DstirSceneDesc), D, D, C.c_int, D, D, D, D, D, D, D, D, C.c_int]
        for name in ('oracle_rollout_f64', 'oracle_rollout_f32', 'oracle_rollout_last_f64'):
            getattr(lib, name).argtypes = sig_roll
            getattr(lib, name).restype = C.c_int
        for name in ('oracle_grad_f64', 'oracle_grad_f32'):
            getattr(lib, name).argtypes = sig_grad
            getattr(lib, name).restype = C.c_int
        lib.oracle_grad_seeded_f64.argtypes = [C.POINTER(DstirSceneDesc), D, D, C.c_int, D, D, D, D, D, D, D, D,
                                               D, C.c_int]
        lib.oracle_grad_seeded_f64.restype = C.c_int
        lib.oracle_svd3_f64.argtypes = [D, D, D, D, C.c_int64]
        lib.oracle_svd3_f64.restype = None
        lib.oracle_svd3_backward_f64.argtypes = [D, D, D, D, D, D, D, C.c_int64]
        lib.oracle_svd3_backward_f64.restype = None
        lib.oracle_max_threads.restype = C.c_int
        _libs[variant] = lib
    return _libs[variant]


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _arr(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def rollout(desc, params, traj, T, x0, v0=None, C0=None, F0=None, precision='f64',
            threads=1, return_states=False, variant=None):
    """Forward rollout; returns (force [T,3], states [(T+1),N,24] or None, status)."""
    lib = load(variant)
    N = desc.n_liquid + desc.n_rod + desc.n_container
    params, traj = _arr(params), _arr(traj)
    x0, v0, C0, F0 = _arr(x0), _arr(v0), _arr(C0), _arr(F0)
    force = np.zeros((T, 3))
    states = np.zeros((T + 1, N, 24)) if return_states else None
    fn = lib.oracle_rollout_f64 if precision == 'f64' else lib.oracle_rollout_f32
    rc = fn(C.byref(desc), _p(params), _p(traj), T, _p(x0), _p(v0), _p(C0), _p(F0),
            _p(force), _p(states), threads)
    if rc < 0:
        raise RuntimeError('oracle rollout failed: %d' % rc)
    return force, states, rc


def grad(desc, params, traj, T, x0, dL_dforce, v0=None, C0=None, F0=None, precision='f64',
         threads=1, want_state0=False, variant=None):
    """Rollout + reverse pass; returns (force, dL_dparams[4], dL_dstate0 [N,24] or None, status)."""
    lib = load(variant)
    N = desc.n_liquid + desc.n_rod + desc.n_container
    params, traj = _arr(params), _arr(traj)
    x0, v0, C0, F0 = _arr(x0), _arr(v0), _arr(C0), _arr(F0)
    dL = _arr(dL_dforce, (T, 3))
    force = np.zeros((T, 3))
    dp = np.zeros(4)
    ds = np.zeros((N, 24)) if want_state0 else None
    fn = lib.oracle_grad_f64 if precision == 'f64' else lib.oracle_grad_f32
    rc = fn(C.byref(desc), _p(params), _p(traj), T, _p(x0), _p(v0), _p(C0), _p(F0),
            _p(dL), _p(force), _p(dp), _p(ds), threads)
    if rc < 0:
        raise RuntimeError('oracle grad failed: %d' % rc)
    return force, dp, ds, rc


def rollout_last(desc, params, traj, T, x0, v0=None, C0=None, F0=None, threads=1):
    """FP64 rollout returning (force [T,3], final state [N,24], status); keeps
    only the states of this call, so long rollouts run as chained segments."""
    lib = load()
    N = desc.n_liquid + desc.n_rod + desc.n_container
    params, traj = _arr(params), _arr(traj)
    x0, v0, C0, F0 = _arr(x0), _arr(v0), _arr(C0), _arr(F0)
    force = np.zeros((T, 3))
    last = np.zeros((N, 24))
    rc = lib.oracle_rollout_last_f64(C.byref(desc), _p(params), _p(traj), T, _p(x0), _p(v0), _p(C0), _p(F0),
                                     _p(force), _p(last), threads)
    if rc < 0:
        raise RuntimeError('oracle rollout failed: %d' % rc)
    return force, last, rc


def grad_seeded(desc, params, traj, T, x0, dL_dforce, dL_dstateT=None, v0=None, C0=None, F0=None, threads=1):
    """FP64 rollout + reverse pass seeded with the adjoint of the final state
    [N,24] (None: zero); returns (force, dL_dparams[4], dL_dstate0 [N,24],
    status).  Chaining it backwards over segments gives the gradient of a
    rollout whose states do not fit in memory at once."""
    lib = load()
    N = desc.n_liquid + desc.n_rod + desc.n_container
    params, traj = _arr(params), _arr(traj)
    x0, v0, C0, F0 = _arr(x0), _arr(v0), _arr(C0), _arr(F0)
    dL = _arr(dL_dforce, (T, 3))
    seed = None if dL_dstateT is None else _arr(dL_dstateT, (N, 24))
    force = np.zeros((T, 3))
    dp = np.zeros(4)
    ds = np.zeros((N, 24))
    rc = lib.oracle_grad_seeded_f64(C.byref(desc), _p(params), _p(traj), T, _p(x0), _p(v0), _p(C0), _p(F0),
                                    _p(dL), _p(seed), _p(force), _p(dp), _p(ds), threads)
    if rc < 0:
        raise RuntimeError('oracle grad failed: %d' % rc)
    return force, dp, ds, rc


def rollout_chain(desc, params, traj, T, x0, K, threads=1, w=None):
    """FP64 rollout of T substeps from rest at positions x0, chained over
    K-substep segments through :func:`rollout_last` (a call keeps every state
    of its substeps, so long rollouts of large scenes run segment by segment).
    Without ``w``: returns the forces [T,3].  With ``w`` = dL/dforce [T,3]:
    also runs the reverse pass segment by segment, last to first, each seeded
    with the state adjoint of the later segment (:func:`grad_seeded`), and
    returns (forces, dL/dparams[4])."""
    x0 = np.asarray(x0, np.float64)
    N = x0.shape[0]
    state = np.zeros((N, 24))
    state[:, 0:3] = x0
    state[:, 15:24] = np.eye(3).reshape(1, 9)
    starts, ckpts, forces = list(range(0, T, K)), [], []
    for s0 in starts:
        L = min(K, T - s0)
        ckpts.append(state)
        f, state, _ = rollout_last(desc, params, traj[s0:s0 + L + 1], L, state[:, 0:3], state[:, 3:6],
                                   state[:, 6:15], state[:, 15:24], threads=threads)
        forces.append(f)
    force = np.concatenate(forces, 0)
    if w is None:
        return force
    w = np.asarray(w, np.float64).reshape(T, 3)
    dp = np.zeros(4)
    seed = None
    for s0, st in reversed(list(zip(starts, ckpts))):
        L = min(K, T - s0)
        _, dps, seed, _ = grad_seeded(desc, params, traj[s0:s0 + L + 1], L, st[:, 0:3], w[s0:s0 + L], seed,
                                      st[:, 3:6], st[:, 6:15], st[:, 15:24], threads=threads)
        dp += dps
    return force, dp


def svd3(A):
    lib = load()
    A = _arr(A).reshape(-1, 9)
    n = A.shape[0]
    U, S, V = np.zeros((n, 9)), np.zeros((n, 3)), np.zeros((n, 9))
    lib.oracle_svd3_f64(_p(A), _p(U), _p(S), _p(V), n)
    return U.reshape(n, 3, 3), S, V.reshape(n, 3, 3)


def svd3_backward(gU, gS, gV, U, S, V):
    lib = load()
    gU, gS, gV = _arr(gU).reshape(-1, 9), _arr(gS).reshape(-1, 3), _arr(gV).reshape(-1, 9)
    U, S, V = _arr(U).reshape(-1, 9), _arr(S).reshape(-1, 3), _arr(V).reshape(-1, 9)
    n = U.shape[0]
    gA = np.zeros((n, 9))
    lib.oracle_svd3_backward_f64(_p(gU), _p(gS), _p(gV), _p(U), _p(S), _p(V), _p(gA), n)
    return gA.reshape(n, 3, 3)


def branch_counts():
    """Counts of the boundary rules taken since the last call (``branch_counts``
    variant, forward substeps of every rollout), as a dict keyed by
    :data:`BRANCHES`; clears them."""
    lib = load('branch_counts')
    lib.oracle_branch_counts.argtypes = [C.POINTER(C.c_longlong), C.c_int]
    lib.oracle_branch_counts.restype = C.c_int
    out = (C.c_longlong * len(BRANCHES))()
    lib.oracle_branch_counts(out, len(BRANCHES))
    return dict(zip(BRANCHES, [int(v) for v in out]))


def max_threads():
    return int(load().oracle_max_threads())
