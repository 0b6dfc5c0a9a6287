"""dstir_substep_static: the substep entry point that allocates nothing.

Callers that may not call cudaMalloc -- for instance code running inside a host
framework that owns the device memory pool, or a stepping loop that cannot
take the synchronisation an allocation may cause -- use this entry point; its
grids and tables live in a static device array inside the library.  This test
calls it through the C ABI twice in a row (substeps 0 and 1, the second one
fed with the output of the first) and compares each result with the handle
based entry point dstir_substep, for a moving-cylinder scene and for the
reference's container + rod-particle scene.  It is kept in its own file so that
pytest collects it last.
"""

import ctypes

import numpy as np
import pytest
import torch

from diffstir_gb300 import _abi
from diffstir_gb300 import scene as S
from diffstir_gb300._lib import lib
from diffstir_gb300.simulator import Simulator

pytestmark = pytest.mark.gpu

RTOL = 1e-5  # both paths run the same kernels; only float atomic ordering differs


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _soa(x, v, C, F):
    """[24][n] component-major state from AoS tensors."""
    n = x.shape[0]
    return torch.cat([x.reshape(n, 3), v.reshape(n, 3), C.reshape(n, 9), F.reshape(n, 9)], 1).t().contiguous()


def _rel(a, b):
    a, b = a.double(), b.double()
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-30))


def _scenes():
    cyl = S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=2, seed=3)
    ref = S.reference_scene(seed=0, n_steps=2, n_liquid=300, n_rod=40, n_container=60, n_grid=32,
                            model=S.MODEL_CARREAU, params=(2.0, 0.1, 0.6, 0.8))
    return [('cylinder', cyl), ('reference', ref)]


@pytest.mark.parametrize('name,sc', _scenes(), ids=lambda v: v if isinstance(v, str) else '')
def test_static_substep_matches_handle_substep_twice(name, sc):
    dev = torch.device('cuda')
    L = lib()
    # existing entry point: handle with library-allocated scratch
    sim = Simulator(sc, max_steps=2)
    f_handle = [sim.substep(0)[0].clone()]
    st1 = sim.get_state()
    f_handle.append(sim.substep(1)[0].clone())
    st2 = sim.get_state()
    # allocation-free entry point, same inputs
    n = sc.n_particles
    x0 = torch.as_tensor(sc.x0(), dtype=torch.float32, device=dev)
    eye = torch.eye(3, device=dev).reshape(1, 9).repeat(n, 1)
    state = _soa(x0, torch.zeros_like(x0), torch.zeros((n, 9), device=dev), eye)
    params = torch.as_tensor(sc.params, dtype=torch.float32, device=dev)
    traj = torch.as_tensor(sc.trajectory, dtype=torch.float32, device=dev)
    desc = sc.desc
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs = []
    for f in range(2):
        nxt = torch.empty_like(state)
        force = torch.empty(3, device=dev)
        traj2 = traj[f:f + 2].contiguous()
        rc = L.dstir_substep_static(ctypes.byref(desc), _ptr(params), _ptr(traj2), _ptr(state), _ptr(nxt),
                                    _ptr(force), stream)
        assert rc == _abi.DSTIR_OK
        outs.append((nxt, force))
        state = nxt
    torch.cuda.synchronize()
    for (nxt, force), st, fh in zip(outs, (st1, st2), f_handle):
        ref_state = _soa(st['x'], st['v'], st['C'], st['F'])
        assert _rel(nxt[0:3], ref_state[0:3]) < RTOL          # x
        assert _rel(nxt[3:6], ref_state[3:6]) < 1e-4          # v
        assert _rel(nxt[6:15], ref_state[6:15]) < 1e-4        # C
        assert _rel(nxt[15:24], ref_state[15:24]) < RTOL      # F
        assert _rel(force, fh) < 1e-4
    sim.close()


def test_static_substep_rejects_oversized_scene():
    sc = S.small_synthetic_scene(n_grid=16, ppc=1, n_steps=1, seed=0)
    d = _abi.DstirSceneDesc()
    ctypes.memmove(ctypes.byref(d), ctypes.byref(sc.desc), ctypes.sizeof(d))
    d.n_grid = 65
    dummy = torch.zeros(16, device='cuda')
    rc = lib().dstir_substep_static(ctypes.byref(d), _ptr(dummy), _ptr(dummy), _ptr(dummy), _ptr(dummy),
                                    _ptr(dummy), None)
    assert rc == _abi.DSTIR_ERANGE
