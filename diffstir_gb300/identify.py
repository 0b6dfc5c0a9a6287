"""Viscosity-parameter identification on top of the batched simulator.

* :func:`adam_identify` runs R random restarts of Adam as ONE batched handle
  (scene replicated R times, one parameter candidate per replica).  Every
  iteration is a single checkpointed forward + adjoint of all R candidates.
* :func:`single_parameter_fitting1` / :func:`magnitude_level` restate the
  reference's magnitude-scaled step rule
  (src/gradient_descent_module.py:3-42), so the reference's driver loop can be
  reproduced on top of :class:`~diffstir_gb300.simulator.Simulator`.
"""

import copy
import math
import os
import time

import numpy as np
import torch

from . import sharding
from .simulator import Simulator

# (K, tau_y, n) bounds of the Herschel-Bulkley identification workload
HB_BOUNDS = {0: (0.1, 2.0), 1: (0.0, 5.0), 2: (0.4, 1.2)}


def force_mse(force, target):
    """Mean squared error of the rod x and z force profiles, per scene [B]."""
    d = (force - target)[..., 0::2]
    return (d * d).mean(dim=(1, 2))


def adam_identify(scene, target, restarts=16, iters=200, lr=1e-2, ckpt_every=50, free=(0, 1, 2), bounds=None,
                  seed=0, options=None, log_every=0, callback=None, state0=None, init_params=None, group=None,
                  shard=None):
    """Fit the parameters ``free`` of ``scene`` to ``target`` [T,3] (or [1,T,3]).

    Parameters are optimised in normalised form u in [0,1] (p = lo + u (hi-lo))
    with torch.optim.Adam(lr), clamped to the box after each step.  Restart 0
    starts from ``init_params`` when given, the others from seeded uniform
    draws.  ``state0`` (dict of x [n,3] and optionally v, C, F of one scene)
    replaces the scene's step-0 state.  Returns a dict with the best
    parameters per restart, the overall best, the loss history [iters, R] and
    the wall time.

    Restarts are independent (each has its own loss, and Adam's update is
    elementwise), so when torch.distributed is initialised (or ``shard`` is
    true) every rank of ``group`` runs the contiguous range
    sharding.shard_range(R, world, rank) of them in its own batched handle,
    with the same initial draws as a single process would give those
    restarts.  Nothing crosses ranks during the iterations; at the end the
    best parameters, best losses and loss histories of all restarts are
    all-gathered, so every rank returns the single-process result.  Then
    ``wall_s`` is the maximum over ranks, ``grad_evals_per_s`` the whole job's
    rate, ``sim`` this rank's handle (None without restarts) and ``callback``
    sees this rank's restarts (global indices ``restart_range``)."""
    bounds = dict(HB_BOUNDS if bounds is None else bounds)
    T = scene.n_steps
    R = int(restarts)
    world, rank = sharding.active(group) if shard is None or shard else (1, 0)
    ra, rb = sharding.shard_range(R, world, rank)
    Rl = rb - ra
    rng = np.random.default_rng(seed)
    free = list(free)
    u0 = rng.uniform(0.05, 0.95, size=(R, len(free)))
    if init_params is not None:
        ip = np.asarray(init_params, dtype=np.float64)
        u0[0] = [np.clip((ip[i] - bounds[i][0]) / (bounds[i][1] - bounds[i][0]), 0.0, 1.0) for i in free]
    sim = None
    hist = np.zeros((iters, Rl))
    best_loss = np.full(Rl, np.inf)
    bp = np.zeros((Rl, 4))
    t0 = time.perf_counter()
    stamps = []
    if Rl > 0:
        scenes = [copy.copy(scene) for _ in range(Rl)]
        sim = Simulator(scenes, max_steps=T, options=options)
        dev = sim.device
        if state0 is not None:
            tile = {k: None if state0.get(k) is None else
                    torch.as_tensor(state0[k], dtype=torch.float32, device=dev).reshape(scene.n_particles,
                                                                                      -1).repeat(Rl, 1)
                    for k in ('x', 'v', 'C', 'F')}
            sim.set_initial_state(tile['x'], tile['v'], tile['C'], tile['F'])
        tgt = torch.as_tensor(np.asarray(target), dtype=torch.float32, device=dev).reshape(1, T, 3).expand(Rl, T, 3)
        lo = torch.tensor([bounds[i][0] for i in free], device=dev)
        hi = torch.tensor([bounds[i][1] for i in free], device=dev)
        u = torch.tensor(u0[ra:rb], dtype=torch.float32, device=dev, requires_grad=True)
        base = torch.as_tensor(np.asarray(scene.params), dtype=torch.float32, device=dev).reshape(1, 4).repeat(Rl, 1)
        opt = torch.optim.Adam([u], lr=lr)
        best_p = base.clone()
        t0 = time.perf_counter()
        for it in range(iters):
            opt.zero_grad()
            p = base.clone()
            p[:, free] = lo + u * (hi - lo)
            force = sim.rollout(p, nsteps=T, ckpt_every=ckpt_every)
            per = force_mse(force, tgt)
            per.sum().backward()
            opt.step()
            with torch.no_grad():
                u.clamp_(0.0, 1.0)
            lv = per.detach().cpu().numpy()
            hist[it] = lv
            better = lv < best_loss
            if better.any():
                best_loss = np.where(better, lv, best_loss)
                idx = torch.as_tensor(np.nonzero(better)[0], device=dev)
                best_p[idx] = p.detach()[idx]
            if log_every and (it % log_every == 0 or it == iters - 1):
                print('iter %4d  loss min %.4e  median %.4e' % (it, lv.min(), np.median(lv)), flush=True)
            if callback is not None:
                callback(it, p.detach(), lv)
            stamps.append(time.perf_counter() - t0)   # lv.cpu() above synchronised
        torch.cuda.synchronize(dev)
        bp = best_p.cpu().numpy().astype(np.float64)
    wall = time.perf_counter() - t0
    # steady rate: iterations after the first (which also sizes the checkpoint buffers)
    if Rl == 0:
        local_rate = 0.0
    elif iters > 1 and stamps[-1] > stamps[0]:
        local_rate = (iters - 1) * Rl / (stamps[-1] - stamps[0])
    else:
        local_rate = iters * Rl / wall
    if world > 1:
        bp = sharding.allgather_rows(torch.as_tensor(bp), R, group).numpy()
        best_loss = sharding.allgather_rows(torch.as_tensor(best_loss), R, group).numpy()
        hist = sharding.allgather_rows(torch.as_tensor(np.ascontiguousarray(hist.T)), R, group).numpy().T
        wall = sharding.max_over_ranks(wall, group)
        rate = sharding.sum_over_ranks(local_rate, group)
    else:
        rate = local_rate
    k = int(np.argmin(best_loss))
    return {'best_params': bp, 'best_loss': best_loss, 'best': bp[k], 'best_index': k, 'history': hist,
            'wall_s': wall, 'grad_evals': iters * R, 'grad_evals_per_s': rate, 'sim': sim,
            'restart_range': (ra, rb)}


def clip_identify(scene, target, frames_per_clip, n_clips=None, carry='x', restarts=8, iters=50, lr=1e-2,
                  ckpt_every=50, free=(0, 1, 2), bounds=None, seed=0, options=None, first_clip_factor=3,
                  log_every=0, group=None, shard=None):
    """Clip-wise identification over a long trajectory, with the state carried
    from clip to clip (the clip loop of src/gradient_descent_module.py:84-139).

    Clip c covers substeps [c*frames_per_clip, (c+1)*frames_per_clip) of
    ``scene.trajectory`` and of ``target`` [T,3].  Each clip is fitted by
    :func:`adam_identify` (restart 0 continues from the previous clip's best
    parameters; the first clip gets ``first_clip_factor`` times the
    iterations, as the reference gives its first clip three times the epochs),
    then rolled forward once with its best parameters to produce the next
    clip's initial state.  ``carry='x'`` carries positions only and restarts
    v, C, F from rest, as the reference does (initial_x.from_numpy of the last
    frame, then initialize_ti_field); ``carry='full'`` carries x, v, C and F.
    Two defects of the reference loop are not reproduced: its ``return`` sits
    inside the clip loop (only clip 0 ever runs), and it loads the window of
    the clip it just finished instead of the next one.

    Under torch.distributed each clip's restarts are sharded over the ranks
    of ``group`` (see :func:`adam_identify`); every rank then knows the best
    parameters, and the roll-forward's final state is taken from rank 0 and
    broadcast, so that all ranks carry the same state into the next clip
    (float atomics make two GPUs' rollouts differ in their last bits).

    Returns a list with one dict per clip (best parameters, best loss, wall
    time, loss history)."""
    from .scene import Scene
    T_all = min(scene.n_steps, np.asarray(target).shape[-2])
    fpc = int(frames_per_clip)
    if n_clips is None:
        n_clips = T_all // fpc
    target = np.asarray(target, dtype=np.float64).reshape(-1, 3)
    state = None
    params = None
    out = []
    for c in range(n_clips):
        t0, t1 = c * fpc, (c + 1) * fpc
        if t1 > T_all:
            break
        sub = Scene(scene.desc, scene.liquid_x, scene.rod_x, scene.container_x, scene.trajectory[t0:t1 + 1],
                    scene.params if params is None else params, dict(scene.info))
        res = adam_identify(sub, target[t0:t1], restarts=restarts,
                            iters=iters * (first_clip_factor if c == 0 else 1), lr=lr, ckpt_every=ckpt_every,
                            free=free, bounds=bounds, seed=seed + c, options=options, state0=state,
                            init_params=params, log_every=log_every, group=group, shard=shard)
        if res['sim'] is not None:
            res['sim'].close()
        params = res['best']
        # roll the clip forward with its best parameters for the next initial state
        sim = Simulator(sub, max_steps=fpc, options=options)
        if state is not None:
            sim.set_initial_state(state['x'], state.get('v'), state.get('C'), state.get('F'))
        sim.set_params(torch.as_tensor(params, dtype=torch.float32).reshape(1, 4))
        sim.forward(fpc)
        st = sim.get_state()
        n = scene.n_particles
        state = {'x': st['x']} if carry == 'x' else {'x': st['x'], 'v': st['v'], 'C': st['C'].reshape(n, 9),
                                                      'F': st['F'].reshape(n, 9)}
        world, _ = sharding.active(group) if shard is None or shard else (1, 0)
        if world > 1:
            state = {k: sharding.broadcast_tensor(v.contiguous(), 0, group) for k, v in state.items()}
        status = sim.status()
        sim.close()
        out.append({'clip': c, 'substeps': (t0, t1), 'best': params.copy(), 'best_loss': float(res['best_loss'].min()),
                    'wall_s': res['wall_s'], 'history': res['history'], 'status': status})
    return out


# ---------------------------------------------------------------------------
# the reference's step rule (src/gradient_descent_module.py:3-42)
# ---------------------------------------------------------------------------
def magnitude_level(a):
    """floor(log10(max(|a|, 1e-11))), NaN -> 0 (gradient_descent_module.py:3-9)."""
    abs_a = max(abs(a), 1e-11)
    lg = math.log10(abs_a)
    if np.isnan(lg):
        lg = 0
    return math.floor(lg)


def single_parameter_fitting1(parameter, parameter_grad, lower_bound, upper_bound, lr, epochs, epoch_index):
    """One magnitude-scaled step of one parameter (gradient_descent_module.py:11-42).

    Returns (new parameter, new learning rate).  Differences from the
    reference: the parameter, bounds and rate are passed in instead of being
    read from module fields, and the bound-halving loop gives up after 2000
    halvings (the reference loops until the step underflows when the bounds
    coincide)."""
    period = epochs - epoch_index
    base = 3
    if abs(parameter_grad) > 0:
        delta = lr * parameter_grad
        new_magnitude = 0
        if parameter_grad < 0:
            new_magnitude = magnitude_level((upper_bound - parameter) / period)
        if parameter_grad > 0:
            new_magnitude = magnitude_level((lower_bound - parameter) / period)
        if epoch_index < 1:
            lr *= pow(base, new_magnitude - magnitude_level(delta))
            delta = lr * parameter_grad
        parameter_update = parameter - delta
        if lower_bound < parameter_update < upper_bound:
            parameter = parameter_update
            lr *= pow(base, new_magnitude - magnitude_level(delta))
        else:
            if parameter_update < lower_bound:
                new_magnitude = magnitude_level((upper_bound - parameter) / period)
            if parameter_update > upper_bound:
                new_magnitude = magnitude_level((lower_bound - parameter) / period)
            lr *= pow(base, new_magnitude - magnitude_level(delta))
            parameter_update = parameter - lr * parameter_grad
            n = 0
            while (parameter_update > upper_bound or parameter_update < lower_bound) and n < 2000:
                lr *= 0.5
                parameter_update = parameter - lr * parameter_grad
                n += 1
            parameter = parameter_update
    return parameter, lr


def main(argv=None):
    """Identification workload from the command line:

        python -m diffstir_gb300.identify --config C5 --restarts 16 --iters 200

    Builds the scene, synthesises the target rod-force profile from seeded
    ground-truth (K, tau_y, n) plus 1% Gaussian noise, runs the batched Adam
    restarts and prints one JSON line with the recovered parameters, their
    relative errors and the wall time."""
    import argparse
    import json

    from . import scene as S

    ap = argparse.ArgumentParser()
    ap.add_argument('--config', default='C5')
    ap.add_argument('--restarts', type=int, default=None)
    ap.add_argument('--iters', type=int, default=200)
    ap.add_argument('--substeps', type=int, default=None)
    ap.add_argument('--lr', type=float, default=1e-2)
    ap.add_argument('--ckpt', type=int, default=None)
    ap.add_argument('--seed', type=int, default=0)
    ap.add_argument('--noise', type=float, default=0.01)
    ap.add_argument('--plain-iters', type=int, default=3,
                    help='iterations of the plain comparison: one restart alone, scalar atomics, no graph')
    ap.add_argument('--frames-per-clip', type=int, default=0,
                    help='> 0: clip-wise identification with the state carried from clip to clip')
    ap.add_argument('--carry', default='x', choices=['x', 'full'])
    ap.add_argument('--autotune', type=int, default=1,
                    help='1: launch options of the batched handle from the autotuner (cached)')
    args = ap.parse_args(argv)
    # under torchrun the restarts are sharded over the ranks, one GPU each
    if int(os.environ.get('WORLD_SIZE', '1')) > 1:
        import torch.distributed as dist
        local = int(os.environ.get('LOCAL_RANK', '0'))
        torch.cuda.set_device(local)
        if not dist.is_initialized():
            dist.init_process_group('nccl', device_id=torch.device('cuda', local))
    world, rank = sharding.active()
    cfg = S.CONFIGS[args.config]
    T = args.substeps or cfg['n_steps']
    R = args.restarts or cfg.get('restarts', 16)
    rng = np.random.default_rng(args.seed)
    truth = S.draw_config_params(args.config, rng)
    sc = S.synthetic_scene(args.config, seed=args.seed, n_steps=T, params=truth)
    sim = Simulator(sc, max_steps=T)
    clean = sim.forward(T)[0].cpu().numpy()
    sim.close()
    target = clean + args.noise * np.abs(clean).mean() * rng.normal(size=clean.shape)
    free = (0, 1, 2) if cfg.get('yield_stress', False) else (0, 2)
    bounds = dict(HB_BOUNDS)
    bounds[2] = tuple(cfg.get('n_range', HB_BOUNDS[2]))   # stay inside the explicitly stable range
    if args.frames_per_clip > 0:
        clips = clip_identify(sc, target, args.frames_per_clip, carry=args.carry, restarts=R, iters=args.iters,
                              lr=args.lr, ckpt_every=args.ckpt or cfg['ckpt'], free=free, bounds=bounds,
                              seed=args.seed + 1)
        out = {'config': args.config, 'particles': sc.n_particles, 'substeps': T, 'restarts': R,
               'iters': args.iters, 'frames_per_clip': args.frames_per_clip, 'carry': args.carry,
               'truth': truth.tolist(),
               'clips': [{'clip': c['clip'], 'substeps': c['substeps'], 'best': c['best'].tolist(),
                          'best_loss': c['best_loss'], 'wall_s': c['wall_s'], 'status': c['status'],
                          'rel_err': {name: float(abs(c['best'][i] - truth[i]) / max(abs(truth[i]), 1e-12))
                                      for name, i in (('K', 0), ('tau_y', 1), ('n', 2)) if i in free}}
                         for c in clips]}
        if rank == 0:
            print(json.dumps(out), flush=True)
        return out
    opts = None
    ra, rb = sharding.shard_range(R, world, rank)
    if args.autotune and rb > ra:
        from . import autotune
        opts = autotune.autotune([copy.copy(sc) for _ in range(rb - ra)])
    res = adam_identify(sc, target, restarts=R, iters=args.iters, lr=args.lr, ckpt_every=args.ckpt or cfg['ckpt'],
                        free=free, bounds=bounds, seed=args.seed + 1, options=opts)
    if res['sim'] is not None:
        res['sim'].close()
    plain = None
    if args.plain_iters > 0 and rank == 0:
        p1 = adam_identify(sc, target, restarts=1, iters=args.plain_iters, lr=args.lr,
                           ckpt_every=args.ckpt or cfg['ckpt'], free=free, bounds=bounds, seed=args.seed + 1,
                           options={'p2g': 0, 'graph': 0, 'fuse': 0, 'fuse_adj': 0}, shard=False)
        p1['sim'].close()
        plain = p1['grad_evals_per_s']
    best = res['best']
    rel = {name: float(abs(best[i] - truth[i]) / max(abs(truth[i]), 1e-12)) for name, i in
           (('K', 0), ('tau_y', 1), ('n', 2)) if i in free}
    out = {'config': args.config, 'particles': sc.n_particles, 'substeps': T, 'restarts': R, 'iters': args.iters,
           'options': opts, 'truth': truth.tolist(), 'best': best.tolist(), 'rel_err': rel,
           'best_loss': float(res['best_loss'].min()), 'initial_loss_min': float(res['history'][0].min()),
           'wall_s': res['wall_s'], 'grad_evals': res['grad_evals'],
           'grad_evals_per_s': res['grad_evals_per_s'], 'plain_grad_evals_per_s': plain,
           'speedup_vs_plain': None if not plain else res['grad_evals_per_s'] / plain, 'ranks': world}
    if rank == 0:
        print(json.dumps(out), flush=True)
    return out


if __name__ == '__main__':
    main()
