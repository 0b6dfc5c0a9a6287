"""Device status word: a non-finite particle state raises DSTIR_STATUS_NAN.

The reference's only handling of non-finite values is a print in its
parameter update (src/gradient_descent_module.py:51-54).  Here the G2P kernel
flags any non-finite new position, velocity or affine matrix in the handle's
status word, which dstir_status reads and clears.  The non-finite value is
injected on the host: a NaN yield stress in the uploaded parameters makes the
Herschel-Bulkley viscosity tau_y / gamma + K gamma^(n-1) NaN, and with it the
stress, the grid momentum and the gathered velocity.  Non-finite positions
stay memory-safe: the stencil base of a NaN coordinate converts to cell 0 and
an infinite one fails the in-grid test.
"""

import numpy as np
import pytest
import torch

from diffstir_gb300 import _abi
from diffstir_gb300 import scene as S
from diffstir_gb300.simulator import Simulator

pytestmark = pytest.mark.gpu


def test_nan_parameter_raises_nan_status_and_clears_on_read():
    T = 10
    sc = S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=1, params=(0.5, 0.2, 0.7, 0.0))
    sim = Simulator(sc, max_steps=T)
    good = torch.tensor(np.asarray(sc.params, np.float32)[None], device='cuda')
    sim.set_params(good)
    sim.reset()
    f = sim.forward(T)
    assert torch.isfinite(f).all()
    assert sim.status() == 0
    bad = good.clone()
    bad[0, 1] = float('nan')  # tau_y
    sim.set_params(bad)
    sim.reset()
    f = sim.forward(T)
    flags = sim.status()
    assert flags & _abi.DSTIR_STATUS_NAN
    assert not torch.isfinite(f).all()
    # reading the word cleared it; a finite rollout leaves it clear
    sim.set_params(good)
    sim.reset()
    f = sim.forward(T)
    assert torch.isfinite(f).all()
    assert sim.status() == 0
    sim.close()


def test_nan_status_from_a_recorded_rollout_and_its_reverse_pass():
    T = 12
    sc = S.small_synthetic_scene(n_grid=16, ppc=2, n_steps=T, seed=2, params=(0.5, 0.2, 0.7, 0.0))
    sim = Simulator(sc, max_steps=T)
    p = torch.tensor(np.asarray(sc.params, np.float32)[None], device='cuda')
    p[0, 1] = float('nan')
    sim.set_params(p)
    sim.reset()
    f = sim.forward(T, ckpt_every=4, record=True)
    dp = sim.backward(torch.ones_like(f))
    assert sim.status() & _abi.DSTIR_STATUS_NAN
    assert not torch.isfinite(dp).all()
    sim.close()
