"""Python-facing simulator over the C ABI (libdiffstir.so).

:class:`Simulator` owns one ``DstirHandle`` holding a batch of scenes on one
GPU.  All arrays crossing the boundary are torch CUDA tensors (float32,
contiguous); the calls are enqueued on torch's current CUDA stream.

:class:`RolloutFunction` is the ``torch.autograd.Function`` over a whole
checkpointed rollout: forward returns the rod force profile, backward returns
d loss / d constitutive parameters (and optionally d loss / d initial state),
which is what ``ti.ad.Tape`` produced for the reference
(src/gradient_descent_module.py:103-120).
"""

import ctypes

import numpy as np
import torch

from . import _abi
from ._lib import check, lib


def _ptr(t):
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev(t, device, shape=None, dtype=torch.float32):
    t = torch.as_tensor(t, dtype=dtype, device=device)
    if shape is not None:
        t = t.reshape(shape)
    return t.contiguous()


class Simulator:
    """A batch of MLS-MPM scenes advanced together.

    ``scenes`` is a :class:`~diffstir_gb300.scene.Scene` or a list of them.
    ``max_steps`` bounds the substeps of one rollout (default: the longest
    trajectory).  ``options`` are passed to ``dstir_set_option`` (``p2g``,
    ``block``, ``graph``).
    """

    def __init__(self, scenes, max_steps=None, device='cuda', options=None, reorder=True):
        if not torch.cuda.is_available():
            raise RuntimeError('diffstir_gb300.Simulator needs a CUDA device (there is no CPU path)')
        if not isinstance(scenes, (list, tuple)):
            scenes = [scenes]
        self.scenes = list(scenes)
        self.device = torch.device(device)
        self.B = len(self.scenes)
        if max_steps is None:
            max_steps = max(s.n_steps for s in self.scenes)
        self.max_steps = int(max_steps)
        descs = (_abi.DstirSceneDesc * self.B)(*[s.desc for s in self.scenes])
        self._lib = lib()
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            torch.cuda.current_stream().synchronize()
            rc = self._lib.dstir_create(descs, self.B, self.max_steps, ctypes.byref(h))
        if rc < 0:
            raise RuntimeError('dstir_create failed: %s' % _abi.errname(rc))
        self._h = h
        self.counts = [s.n_particles for s in self.scenes]
        self.N = int(sum(self.counts))
        self.offsets = np.concatenate([[0], np.cumsum(self.counts)]).astype(np.int64)
        for k, v in (options or {}).items():
            self.set_option(k, v)
        x0 = np.concatenate([s.x0() for s in self.scenes], 0)
        # internal particle order: position q of the handle holds caller particle perm[q]
        self._perm = interleaved_order(self.scenes, x0) if reorder else np.arange(self.N)
        self._perm_t = torch.from_numpy(self._perm).to(self.device)
        self._inv_t = torch.empty_like(self._perm_t)
        self._inv_t[self._perm_t] = torch.arange(self.N, device=self.device)
        self.set_x0(x0)
        self.set_params(np.stack([s.params for s in self.scenes]),
                        [s.desc.model for s in self.scenes])
        self.set_trajectories([s.trajectory for s in self.scenes])

    # -- lifetime ----------------------------------------------------------
    def close(self):
        if getattr(self, '_h', None) is not None and self._h.value:
            torch.cuda.synchronize(self.device)
            self._lib.dstir_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        return check(rc, self._h, what)

    # -- configuration -----------------------------------------------------
    def set_option(self, key, value):
        self._check(self._lib.dstir_set_option(self._h, key.encode(), int(value)), 'set_option')

    def get_option(self, key):
        v = ctypes.c_int64()
        self._check(self._lib.dstir_get_option(self._h, key.encode(), ctypes.byref(v)), 'get_option')
        return v.value

    def _to_internal(self, t, shape):
        return None if t is None else _dev(t, self.device, shape)[self._perm_t].contiguous()

    def _to_caller(self, t):
        return t[self._inv_t]

    def set_x0(self, x0):
        """Step-0 positions (caller order) used by :meth:`reset`; resets."""
        self._x0 = self._to_internal(x0, (self.N, 3))
        self._init = (self._x0, None, None, None)
        self.reset()

    def set_initial_state(self, x, v=None, C=None, F=None):
        """State (caller order) that :meth:`reset` restores from now on, for a
        rollout that continues an earlier one (the next clip of a long
        trajectory); v/C default to zero and F to identity, as in
        :meth:`set_state`.  Resets."""
        self._x0 = self._to_internal(x, (self.N, 3))
        self._init = (self._x0, self._to_internal(v, (self.N, 3)), self._to_internal(C, (self.N, 9)),
                      self._to_internal(F, (self.N, 9)))
        self.reset()

    def set_state(self, x, v=None, C=None, F=None):
        """State of all particles in the caller's order (scene-major,
        [liquid|rod|container]); v/C default to zero, F to identity."""
        self._set_state_internal(self._to_internal(x, (self.N, 3)), self._to_internal(v, (self.N, 3)),
                                 self._to_internal(C, (self.N, 9)), self._to_internal(F, (self.N, 9)))

    def _set_state_internal(self, x, v=None, C=None, F=None):
        d = self.device
        x = _dev(x, d, (self.N, 3))
        v = None if v is None else _dev(v, d, (self.N, 3))
        C = None if C is None else _dev(C, d, (self.N, 9))
        F = None if F is None else _dev(F, d, (self.N, 9))
        self._keep = (x, v, C, F)
        self._check(self._lib.dstir_set_state(self._h, _ptr(x), _ptr(v), _ptr(C), _ptr(F), _stream()),
                    'set_state')

    def reset(self):
        """Restore the scenes' step-0 state (x0, v=0, C=0, F=I), as
        initialize_ti_field does (simulation_functions.py:301-319), or the
        state given to :meth:`set_initial_state`."""
        self._set_state_internal(*self._init)

    def get_state(self):
        """Current state in the caller's particle order."""
        d = self.device
        out = {k: torch.empty((self.N, 3) if k in 'xv' else (self.N, 3, 3), device=d) for k in 'xvCF'}
        self._check(self._lib.dstir_get_state(self._h, _ptr(out['x']), _ptr(out['v']), _ptr(out['C']),
                                              _ptr(out['F']), _stream()), 'get_state')
        return {k: self._to_caller(t) for k, t in out.items()}

    def set_params(self, params, models=None):
        p = _dev(params, self.device, (self.B, 4))
        m = None if models is None else _dev(models, self.device, (self.B,), torch.int32)
        self._params_keep = (p, m)
        self._check(self._lib.dstir_set_params(self._h, _ptr(p), _ptr(m), _stream()), 'set_params')

    def set_trajectories(self, trajs):
        T1 = self.max_steps + 1
        buf = np.zeros((self.B, T1, 3), dtype=np.float32)
        for b, t in enumerate(trajs):
            t = np.asarray(t, dtype=np.float64)
            n = min(T1, t.shape[0])
            buf[b, :n] = t[:n]
            if n < T1:
                buf[b, n:] = t[n - 1]
        tt = torch.from_numpy(buf).to(self.device)
        self._traj_keep = tt
        self._check(self._lib.dstir_set_trajectory(self._h, _ptr(tt), _stream()), 'set_trajectory')

    # -- stepping ----------------------------------------------------------
    def forward(self, nsteps, t0=0, ckpt_every=50, record=False, force_out=None):
        """Advance ``nsteps`` substeps; returns the force profile [B, nsteps, 3]."""
        if force_out is None:
            force_out = torch.empty((self.B, nsteps, 3), device=self.device)
        self._check(self._lib.dstir_forward(self._h, int(t0), int(nsteps), int(ckpt_every), int(bool(record)),
                                            _ptr(force_out), _stream()), 'forward')
        return force_out

    def substep(self, f):
        out = torch.empty((self.B, 3), device=self.device)
        self._check(self._lib.dstir_substep(self._h, int(f), _ptr(out), _stream()), 'substep')
        return out

    def backward(self, dL_dforce, want_state0=False):
        """Reverse pass of the last recorded forward.  Returns dL/dparams [B,4]
        (and a dict of dL/d step-0 state when ``want_state0``)."""
        g = _dev(dL_dforce, self.device)
        dp = torch.empty((self.B, 4), device=self.device)
        st = {}
        if want_state0:
            st = {k: torch.empty((self.N, 3) if k in 'xv' else (self.N, 3, 3), device=self.device) for k in 'xvCF'}
        self._check(self._lib.dstir_backward(self._h, _ptr(g), _ptr(dp), _ptr(st.get('x')), _ptr(st.get('v')),
                                             _ptr(st.get('C')), _ptr(st.get('F')), _stream()), 'backward')
        if want_state0:
            return dp, {k: self._to_caller(t) for k, t in st.items()}
        return dp

    def status(self):
        f = ctypes.c_uint32()
        self._check(self._lib.dstir_status(self._h, ctypes.byref(f), _stream()), 'status')
        return f.value

    # -- autograd ----------------------------------------------------------
    def rollout(self, params, nsteps=None, t0=0, ckpt_every=50, reset=True):
        """Differentiable rollout: force [B, nsteps, 3] as a function of
        ``params`` [B, 4] (a torch tensor that may require grad).  With
        ``reset`` the scenes restart from their step-0 state."""
        nsteps = self.max_steps - t0 if nsteps is None else nsteps
        return RolloutFunction.apply(params, self, int(t0), int(nsteps), int(ckpt_every), bool(reset))


class RolloutFunction(torch.autograd.Function):
    """force = rollout(params); grad = adjoint of the checkpointed rollout."""

    @staticmethod
    def forward(ctx, params, sim, t0, nsteps, ckpt_every, reset):
        if reset:
            sim.reset()
        sim.set_params(params.detach())
        force = sim.forward(nsteps, t0=t0, ckpt_every=ckpt_every, record=True)
        ctx.sim = sim
        return force

    @staticmethod
    def backward(ctx, dforce):
        dp = ctx.sim.backward(dforce.contiguous())
        return dp, None, None, None, None, None


def interleaved_order(scenes, x0):
    """Particle order used inside the handle.

    Within each scene and particle kind, particles are sorted by stencil-base
    cell row (i, j), then by their rank inside their cell, then by k.  A warp
    of 32 consecutive particles then covers up to 32 consecutive cells of one
    row, so each of its stencil-node atomics and gathers touches 32
    consecutive grid nodes instead of ~4 nodes 8 times over.  The kernels do
    not depend on the order; it only shapes the memory access pattern.
    Returns perm with internal position q holding caller particle perm[q]."""
    perm = np.empty(x0.shape[0], dtype=np.int64)
    off = 0
    for sc in scenes:
        n = sc.desc.n_grid
        for cnt in (sc.desc.n_liquid, sc.desc.n_rod, sc.desc.n_container):
            idx = np.arange(off, off + cnt)
            if cnt:
                b = np.clip(np.trunc(x0[idx] * n - 0.5), 0, n - 1).astype(np.int64)
                cell = (b[:, 0] * n + b[:, 1]) * n + b[:, 2]
                o = np.argsort(cell, kind='stable')
                cs = cell[o]
                start = np.r_[0, np.nonzero(np.diff(cs))[0] + 1]
                run = np.repeat(start, np.diff(np.r_[start, cnt]))
                rank = np.empty(cnt, dtype=np.int64)
                rank[o] = np.arange(cnt) - run
                order = np.lexsort((b[:, 2], rank, b[:, 1], b[:, 0]))
                perm[off:off + cnt] = idx[order]
            off += cnt
    return perm


def stack_batch(scenes, max_steps=None, **kw):
    return Simulator(scenes, max_steps=max_steps, **kw)
