#!/usr/bin/env python
"""Throughput benchmark of the differentiable MLS-MPM stirring path on GB300.

One step = one gradient evaluation of the identification loss: a recorded
forward rollout (rod force profile) followed by the checkpointed adjoint,
giving d loss / d viscosity parameters.  Default workload (one GPU): the 64^3
single-scene configuration, 8 particles per cell (~604k particles), 2000
substeps, checkpoint every 50, power-law fluid, rod moving on a circle.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  ``value`` is particle-substeps/s of forward +
adjoint with inputs resident in HBM; ``e2e`` is the same metric through the
public Python API with host (pinned) inputs copied in and results copied out
every step.  ``--impl reference`` times the CPU restatement of the reference
(oracle/, FP32, all host threads) on a bounded sample of the same workload.
"""

import argparse
import glob
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'grad evals/s & particle-substeps/s, batched adjoint vs plain on GB300 @ grad err≤1e-3'
UNIT = 'particle-substeps/s'

# Algorithmic bytes of each kernel: (bytes per liquid particle, bytes per grid node)
# p2g: read x,v,C,F (96) write F (36); grid result 16/node
# grid: read P,M (16) write v (12) clear P,M (16)
# g2p: read x (12) write x,v,C (60); read v grid 12/node
# g2p_adj: read x (12), adj x,v,C (60), write adj x (12); read v 12, write grid adjoint 12 per node
# grid_adj: read P,M 16, grid adjoint 12, write P/M adjoint 16, clear 12
# p2g_adj: read state 96, adj F 36, adj x 12, write adj state 96; read P/M adjoint 16 per node
# g2p_p2g (G2P of substep f fused with P2G of f+1): read x (12), F (36), write
#   x,v,C (60), F (36); read v grid 12/node, P2G result 16/node
KERNEL_BYTES = {
    'p2g': (132, 16), 'grid': (0, 44), 'g2p': (72, 12),
    'g2p_adj': (84, 24), 'grid_adj': (0, 56), 'p2g_adj': (240, 16),
    'g2p_p2g': (144, 28),
    # p2g_adj_g2p_adj (P2G adjoint of f fused with the G2P adjoint of f-1): read
    #   state f (96), adj F (36), adj x part (12), x of f-1 (12); write adj F (36),
    #   adj x part of f-1 (12); read P/M adjoint 16 + velocity 12, write grid adjoint 12 per node
    'p2g_adj_g2p_adj': (204, 40),
}
KERNELS = ['p2g', 'grid', 'g2p', 'g2p_adj', 'grid_adj', 'p2g_adj', 'bin', 'g2p_p2g', 'p2g_adj_g2p_adj', 'other',
           'p2g_rc', 'grid_rc', 'g2p_rc', 'bin_rc', 'g2p_p2g_rc', 'seg_fwd', 'seg_adj', 'seg_fwd_rc']
# the in-library profiler reports the reverse pass's segment recompute under
# <kernel>_rc; the roofline counts both launches of the same kernel together
RC = {'p2g': 'p2g_rc', 'grid': 'grid_rc', 'g2p': 'g2p_rc', 'g2p_p2g': 'g2p_p2g_rc'}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--config', default='C2')
    ap.add_argument('--substeps', type=int, default=None, help='override the substep count')
    ap.add_argument('--ckpt', type=int, default=None)
    ap.add_argument('--batch', type=int, default=None, help='scenes per GPU (default: the configuration\'s)')
    ap.add_argument('--p2g', type=int, default=None,
                    help='0 scalar atomics, 1 vector atomics, 3 brick tiles, 4 warp-aggregated vector atomics')
    ap.add_argument('--graph', type=int, default=None, help='1: replay rollouts as CUDA graphs')
    ap.add_argument('--block', type=int, default=None)
    ap.add_argument('--gblock', type=int, default=None)
    ap.add_argument('--autotune', type=int, default=1, help='1: launch options from the autotuner (cached)')
    ap.add_argument('--brick-scatter', type=int, default=None, help='brick P2G scatter: 0 atom, 1 red.shared, 2 global')
    ap.add_argument('--brick-gather', type=int, default=None)
    ap.add_argument('--fuse', type=int, default=None, help='1: G2P(f) fused with P2G(f+1)')
    ap.add_argument('--fuse-adj', type=int, default=None, help='1: P2G adjoint of f fused with G2P adjoint of f-1')
    ap.add_argument('--resort', type=int, default=None, help='1: re-sort the particle order at every checkpoint')
    ap.add_argument('--tight', type=int, default=None, help='register-cap level of the particle kernels: 0..3')
    ap.add_argument('--box', type=int, default=None, help='1: grid kernels skip nodes outside the occupied box')
    ap.add_argument('--store-grids', type=int, default=None, help='1: keep every substep\'s grids, recompute states only')
    ap.add_argument('--overlap', type=int, default=None, help='1: segment recompute on a second stream')
    ap.add_argument('--lsort', type=int, default=None, help='1: re-interleave each block before the warp scatters')
    ap.add_argument('--pdl', type=int, default=None, help='1: programmatic dependent launch of the substep kernels')
    ap.add_argument('--lstage', type=int, default=None, help='re-interleaved blocks stage their state in shared memory (bits: P2G, G2P adjoint)')
    ap.add_argument('--gprio', type=int, default=None, help='grid kernels at the greatest launch priority')
    ap.add_argument('--prefetch', type=int, default=None, help='adjoint blocks hint L2 for the block this many later')
    ap.add_argument('--persist', type=int, default=None, help='1: persistent cooperative launches per chunk / segment')
    ap.add_argument('--cpu-sample', type=int, default=24, help='substeps in the CPU baseline sample')
    ap.add_argument('--ref-sample', type=int, default=12, help='substeps per reference-arm step')
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-fd', action='store_true', help='skip the central-difference gradient check')
    ap.add_argument('--no-plain', action='store_true', help='skip the plain single-scene comparison')
    ap.add_argument('--no-kept', action='store_true', help='skip the kept-grids measurement')
    ap.add_argument('--fd-h', type=float, default=1e-3, help='relative step of the gradient check')
    ap.add_argument('--no-fp64', action='store_true', help='skip the FP64 oracle gradient check')
    ap.add_argument('--fp64-substeps', type=int, default=400, help='horizon of the FP64 oracle gradient check')
    ap.add_argument('--no-batched', action='store_true', help='skip the batched 64-scene leg')
    ap.add_argument('--batched-config', default='C3', help='configuration of the batched leg')
    ap.add_argument('--batched-steps', type=int, default=2, help='timed gradient evaluations of the batched leg')
    ap.add_argument('--plain-evals', type=int, default=3, help='timed gradient evaluations of the plain leg')
    return ap.parse_args()


# ---------------------------------------------------------------------------
def dist_setup(args):
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix='.csv')
            os.close(fd)
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.Q,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(',')]
            if len(parts) < 9:
                continue
            try:
                rows.append(parts)
            except Exception:
                pass
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace('.', '', 1).isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace('.', '', 1).isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == 'active'})
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': max(mx) if mx else None,
                'reasons': reasons, 'samples': len(rows)}


def peaks():
    try:
        p = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json')))
        return float(p['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


def ncu_value(name, kernel, workload):
    """`name[kernel@workload] = value` from the committed ncu summaries, if any."""
    for path in glob.glob(os.path.join(ROOT, 'profiles', '*.md')) + glob.glob(os.path.join(ROOT, 'profiles', '*.txt')):
        txt = open(path).read()
        m = re.search(r'%s\[%s@%s\]\s*[:=]\s*([0-9.eE+]+)' % (re.escape(name), re.escape(kernel), re.escape(workload)),
                      txt)
        if m:
            return float(m.group(1))
    return None


def ncu_traffic(kernel, workload):
    """dram bytes per launch of `kernel` from the committed ncu summary, if any."""
    return ncu_value('traffic_bytes_per_launch', kernel, workload)


def fp32_peak():
    """FP32 FMA flop/s this GPU sustains (dstir_measure_fp32_rate), or None."""
    import ctypes
    import torch
    from diffstir_gb300 import _lib
    rate = ctypes.c_double(0.0)
    torch.cuda.synchronize()
    rc = _lib.lib().dstir_measure_fp32_rate(20000, ctypes.byref(rate),
                                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rate.value if rc == 0 else None


def red_peak(G):
    """Vector-RED sectors/s this GPU retires on a grid of G nodes
    (dstir_measure_red_rate), or None."""
    import ctypes
    import torch
    from diffstir_gb300 import _lib
    rate = ctypes.c_double(0.0)
    torch.cuda.synchronize()
    rc = _lib.lib().dstir_measure_red_rate(max(int(G), 1 << 18), 256, ctypes.byref(rate),
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rate.value if rc == 0 else None


def build_workload(args, rank):
    """Scenes of this rank: one for the single-scene configurations, ``batch``
    seeded scenes (uneven fill heights) for the batched one."""
    from diffstir_gb300 import scene as S
    cfg = S.CONFIGS[args.config]
    T = args.substeps or cfg['n_steps']
    B = args.batch or cfg.get('batch', 1)
    scenes = [S.synthetic_scene(args.config, seed=rank * B + b, n_steps=T) for b in range(B)]
    ckpt = args.ckpt or cfg['ckpt']
    return scenes, T, ckpt


def workload_name(args, scenes, T, ckpt):
    d = scenes[0].desc
    N = sum(s.n_particles for s in scenes)
    visc = 'Herschel-Bulkley fluid' if S_yield(args.config) else 'power-law fluid'
    if len(scenes) == 1:
        return ('%s: %d^3 grid, %d particles (8/cell), %d substeps, checkpoint every %d, %s, '
                'moving cylinder rod; forward + checkpointed adjoint' % (args.config, d.n_grid, N, T, ckpt, visc))
    return ('%s: %d scenes of %d^3 grid, %d particles in all (%d..%d per scene), %d substeps, checkpoint every %d, '
            '%s, moving cylinder rod; batched forward + checkpointed adjoint' %
            (args.config, len(scenes), d.n_grid, N, min(s.n_particles for s in scenes),
             max(s.n_particles for s in scenes), T, ckpt, visc))


def S_yield(config):
    from diffstir_gb300 import scene as S
    return bool(S.CONFIGS[config].get('yield_stress', False))


# ---------------------------------------------------------------------------
def cpu_sample(sc, T_sample, threads):
    """Oracle FP32 forward + adjoint of the first T_sample substeps."""
    import oracle
    T = T_sample
    w = np.zeros((T, 3))
    w[:, 0] = w[:, 2] = 1.0 / T
    t0 = time.perf_counter()
    oracle.grad(sc.desc, sc.params, sc.trajectory[:T + 1], T, sc.x0(), w, precision='f32', threads=threads)
    return time.perf_counter() - t0


def fp64_grad_check(sc, p32, target32, Ts, norm, gpu_dp, free, names, h_rel, threads, K=50):
    """The GPU adjoint of scene 0's force loss over the first Ts substeps
    against the FP64 oracle: its adjoint (the reverse pass of the oracle's
    FP64 rollout) and its central differences at h = h_rel x |param|.  The
    oracle runs on the same float32 inputs the GPU got."""
    t0 = time.perf_counter()
    desc = sc.desc
    x0 = np.asarray(sc.x0(), np.float32).astype(np.float64)
    traj = np.asarray(sc.trajectory[:Ts + 1], np.float32).astype(np.float64)
    p = np.asarray(p32, np.float32).astype(np.float64)
    tgt = np.asarray(target32, np.float64)[:Ts]

    def loss_of(force):
        d = (force - tgt)[:, 0::2]
        return float((d * d).sum() / norm)

    import oracle
    f64 = oracle.rollout_chain(desc, p, traj, Ts, x0, K, threads)
    w = np.zeros((Ts, 3))
    w[:, 0::2] = 2.0 * (f64 - tgt)[:, 0::2] / norm
    _, dp64 = oracle.rollout_chain(desc, p, traj, Ts, x0, K, threads, w)
    out = {'what': 'GPU adjoint (FP32) of scene 0 against the FP64 oracle over the first %d substeps: the '
                   'oracle\'s own reverse pass, and its central differences at h = %g x |param|' % (Ts, h_rel),
           'substeps': Ts, 'threads': threads, 'gpu_adjoint': {}, 'fp64_adjoint': {}, 'fp64_fd': {},
           'rel_err_gpu_vs_fp64_adjoint': {}, 'rel_err_gpu_vs_fp64_fd': {}, 'rel_err_fp64_adjoint_vs_fd': {}}
    for i in free:
        h = h_rel * max(abs(p[i]), 1e-3)
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (loss_of(oracle.rollout_chain(desc, pp, traj, Ts, x0, K, threads)) -
              loss_of(oracle.rollout_chain(desc, pm, traj, Ts, x0, K, threads))) / (2.0 * h)
        g, a = float(gpu_dp[i]), float(dp64[i])
        nm = names[i]
        out['gpu_adjoint'][nm], out['fp64_adjoint'][nm], out['fp64_fd'][nm] = g, a, fd
        out['rel_err_gpu_vs_fp64_adjoint'][nm] = abs(g - a) / max(abs(a), 1e-30)
        out['rel_err_gpu_vs_fp64_fd'][nm] = abs(g - fd) / max(abs(fd), 1e-30)
        out['rel_err_fp64_adjoint_vs_fd'][nm] = abs(a - fd) / max(abs(fd), 1e-30)
    out['rel_err_max'] = max(max(out['rel_err_gpu_vs_fp64_adjoint'].values()),
                             max(out['rel_err_gpu_vs_fp64_fd'].values()))
    out['seconds'] = time.perf_counter() - t0
    return out


def plain_leg(scenes, targets, params, T, ckpt, n_evals, stream):
    """The reference's algorithm on the GPU, one scene at a time: per-particle
    scalar float atomics, particles in generation order, no graph.  Times one
    gradient evaluation of each of ``n_evals`` scenes (cycling through
    ``scenes``) after an untimed one."""
    import torch
    from diffstir_gb300.simulator import Simulator
    sims = {}
    evals = [(i % len(scenes)) for i in range(n_evals)]

    def one(i):
        if i not in sims:
            sims[i] = Simulator([scenes[i]], max_steps=T, options={'p2g': 0, 'graph': 0, 'fuse': 0, 'fuse_adj': 0},
                                reorder=False)
        ps = sims[i]
        ps.set_params(params[i:i + 1].contiguous())
        ps.reset()
        f = ps.forward(T, ckpt_every=ckpt, record=True)
        diff = (f - targets[i:i + 1])[..., 0::2]
        dF = torch.zeros_like(f)
        dF[..., 0::2] = 2.0 * diff / diff.numel()
        return ps.backward(dF)

    one(evals[0])
    for i in set(evals):
        if i not in sims:
            one(i)
    torch.cuda.synchronize()
    q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    q0.record(stream)
    for i in evals:
        one(i)
    q1.record(stream)
    torch.cuda.synchronize()
    ms = q0.elapsed_time(q1)
    for ps in sims.values():
        ps.close()
    n_ps = sum(scenes[i].n_particles for i in evals) * T
    return {'grad_evals_per_s': n_evals * 1e3 / ms, 'value': n_ps / (ms / 1e3), 'unit': UNIT,
            'ms_per_grad_eval': ms / n_evals, 'timed_grad_evals': n_evals,
            'scenes': sorted(set(evals)), 'particles': [scenes[i].n_particles for i in sorted(set(evals))],
            'what': 'one scene at a time, scalar atomics, generation order, no graph; %d timed gradient '
                    'evaluations' % n_evals}


def batched_leg(args, rank, world, dev, stream):
    """The batched workload (64 scenes of 64^3 with uneven fill heights and
    Herschel-Bulkley parameters, 1000 substeps): gradient evaluations of all
    scenes in one handle, against the plain single-scene GPU rollout of the
    same scenes."""
    import torch
    from diffstir_gb300 import scene as S
    from diffstir_gb300 import autotune
    from diffstir_gb300.simulator import Simulator
    cfg = S.CONFIGS[args.batched_config]
    T, ckpt, B = cfg['n_steps'], cfg['ckpt'], cfg.get('batch', 1)
    t_build = time.perf_counter()
    scenes = [S.synthetic_scene(args.batched_config, seed=rank * B + b, n_steps=T) for b in range(B)]
    # the tuner's candidates that win for batches of 64^3 scenes
    opts = autotune.autotune(scenes, candidates=[c for c in autotune.CANDIDATES
                                                 if c.get('p2g') == 4 and c.get('tight') in (2, 3)])
    sim = Simulator(scenes, max_steps=T, options=opts)
    rng = np.random.default_rng(2000 + rank)
    true_p = torch.tensor(np.stack([S.draw_config_params(args.batched_config, rng) for _ in range(B)]),
                          dtype=torch.float32, device=dev)
    sim.set_params(true_p)
    sim.reset()
    target = sim.forward(T).clone()
    params = torch.tensor(np.stack([s.params for s in scenes]), dtype=torch.float32, device=dev)
    build_s = time.perf_counter() - t_build

    def grad_eval():
        sim.set_params(params)
        sim.reset()
        f = sim.forward(T, ckpt_every=ckpt, record=True)
        diff = (f - target)[..., 0::2]
        dF = torch.zeros_like(f)
        dF[..., 0::2] = 2.0 * diff / diff.numel()
        return sim.backward(dF)

    grad_eval()
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.batched_steps):
        grad_eval()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.batched_steps
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    st = sim.status()
    N = sum(s.n_particles for s in scenes)
    opt_used = {k: sim.get_option(k) for k in ('p2g', 'gblock', 'tight', 'lsort', 'lstage', 'pdl', 'overlap')}
    sim.close()
    del sim
    torch.cuda.empty_cache()
    plain = plain_leg(scenes, target, params, T, ckpt, max(args.plain_evals, 3), stream)
    ge = world * B * 1e3 / ms
    return {'workload': '%s: %d scenes of %d^3 grid, %d particles in all (%d..%d per scene), %d substeps, '
                        'checkpoint every %d, Herschel-Bulkley fluid; forward + checkpointed adjoint of all scenes '
                        'per step' % (args.batched_config, B, cfg['n_grid'], N, min(s.n_particles for s in scenes),
                                      max(s.n_particles for s in scenes), T, ckpt),
            'grad_evals_per_s': ge, 'value': world * N * T / (ms / 1e3), 'unit': UNIT, 'ms_per_step': ms,
            'timed_steps': args.batched_steps, 'options': opt_used, 'status_flags': int(st),
            'setup_s': build_s, 'plain': plain,
            'batched_over_plain': {'grad_evals_per_s': ge / plain['grad_evals_per_s'],
                                   'particle_substeps_per_s': world * N * T / (ms / 1e3) / plain['value']}}


def run_reference(args):
    world, rank, local = dist_setup(args)
    if rank != 0:
        return 0
    import oracle
    oracle.build()
    scenes, T, ckpt = build_workload(args, 0)
    sc = scenes[0]
    threads = os.cpu_count() or 1
    Ts = min(args.ref_sample, T)
    for _ in range(args.warmup):
        cpu_sample(sc, Ts, threads)
    times = [cpu_sample(sc, Ts, threads) for _ in range(args.steps)]
    dt = sum(times) / len(times)
    val = sc.n_particles * Ts / dt
    line = {
        'metric': METRIC, 'value': val, 'unit': UNIT, 'n_gpus': args.gpus, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': dt * 1e3, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
        'impl': 'reference',
        'config': {'workload': workload_name(args, scenes, T, ckpt), 'parallelism': 'host threads'},
        'cpu_baseline': {'value': val, 'unit': UNIT, 'cores': threads, 'kind': 'port',
                         'sample': 'first %d of %d substeps of scene 0, forward + adjoint, per step' % (Ts, T)},
        'e2e': {'value': val, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
        'note': 'the reference is a Taichi program (Taichi is not installable offline); its CPU path is '
                'timed through the line-by-line C++ restatement oracle/oracle.cpp (FP32, OpenMP)',
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    world, rank, local = dist_setup(args)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl', device_id=torch.device('cuda', local))
    torch.cuda.set_device(local)
    from diffstir_gb300.simulator import Simulator
    from diffstir_gb300 import scene as S

    scenes, T, ckpt = build_workload(args, rank)
    sc = scenes[0]
    opts = {}
    keys = ('p2g', 'graph', 'block', 'gblock', 'brick_scatter', 'brick_gather', 'fuse', 'fuse_adj', 'resort', 'tight',
            'box', 'store_grids', 'overlap', 'lsort', 'pdl', 'lstage', 'gprio', 'prefetch', 'persist')
    explicit = any(getattr(args, k) is not None for k in keys)
    if args.autotune and not explicit:
        from diffstir_gb300 import autotune
        opts = autotune.autotune(scenes)
    for k in keys:
        if getattr(args, k) is not None:
            opts[k] = getattr(args, k)
    sim = Simulator(scenes, max_steps=T, options=opts)
    dev = torch.device('cuda', local)
    N = sum(s.n_particles for s in scenes)
    B = len(scenes)
    G_all = sum(s.desc.n_grid ** 3 for s in scenes)
    rng = np.random.default_rng(1000 + rank)
    ys = S_yield(args.config)

    # target force profiles from seeded ground-truth parameters
    true_p = torch.tensor(np.stack([S.draw_config_params(args.config, rng) for _ in range(B)]), dtype=torch.float32,
                          device=dev)
    sim.set_params(true_p)
    sim.reset()
    target = sim.forward(T).clone()
    params = torch.tensor(np.stack([s.params for s in scenes]), dtype=torch.float32, device=dev)

    def grad_eval(p):
        sim.set_params(p)
        sim.reset()
        f = sim.forward(T, ckpt_every=ckpt, record=True)
        diff = (f - target)[..., 0::2]
        loss = (diff * diff).mean()
        dF = torch.zeros_like(f)
        dF[..., 0::2] = 2.0 * diff / diff.numel()
        dp = sim.backward(dF)
        return loss, dp

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(args.warmup):
        grad_eval(params)
    torch.cuda.synchronize()
    st = sim.status()

    clocks = ClockSampler(local)
    clocks.start()
    sim.set_option('launches', 0)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        loss, dp = grad_eval(params)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1) / args.steps
    launches = sim.get_option('launches')
    clk = clocks.stop()
    # per-kernel CUDA-event times: one more identical step with every launch
    # bracketed by events on the launching stream (kept out of the timed steps,
    # whose value the event records would perturb for small scenes; graph
    # replay is switched off for this pass so that each launch is visible)
    # A second pass runs with the overlap of the reverse pass off, so that
    # each kernel's mean launch time is not inflated by kernels of the other
    # stream queued beside it; the roofline uses that pass.
    graph_was = sim.get_option('graph')
    overlap_was = sim.get_option('overlap')
    sim.set_option('graph', 0)

    def profiled_pass():
        sim.set_option('profile', 1)
        grad_eval(params)
        torch.cuda.synchronize()
        pr = {k: (sim.get_option('prof_ns:' + k) / 1e6, sim.get_option('prof_count:' + k)) for k in KERNELS}
        sim.set_option('profile', 0)
        return pr

    prof_ovl = profiled_pass()
    sim.set_option('overlap', 0)
    prof = profiled_pass()
    sim.set_option('overlap', overlap_was)
    sim.set_option('graph', graph_was)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        n_all = torch.tensor([float(N)], device=dev)
        dist.all_reduce(n_all)
        n_total = float(n_all.item())
    else:
        n_total = float(N)
    value = n_total * T / (ms / 1e3)

    # the same gradient evaluation with every substep's grids kept (option
    # store_grids: the reverse pass recomputes states with G2P alone), where
    # they fit in a third of the free device memory; reported beside the
    # headline value, which recomputes each segment in full
    kept = None
    grid_bytes = T * G_all * 32
    if not args.no_kept and not sim.get_option('store_grids') and grid_bytes < torch.cuda.mem_get_info(dev)[0] / 3:
        sim.set_option('store_grids', 1)
        for _ in range(2):
            grad_eval(params)
        torch.cuda.synchronize()
        k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k0.record(stream)
        for _ in range(args.steps):
            grad_eval(params)
        k1.record(stream)
        torch.cuda.synchronize()
        kms = k0.elapsed_time(k1) / args.steps
        if world > 1:
            import torch.distributed as dist
            t = torch.tensor([kms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            kms = float(t.item())
        sim.set_option('store_grids', 0)
        kept = {'value': n_total * T / (kms / 1e3), 'unit': UNIT, 'ms_per_step': kms, 'grid_memory_gb': grid_bytes / 1e9,
                'what': 'option store_grids: P2G and velocity grids of all substeps kept; the reverse pass '
                        'recomputes the states of each 50-substep segment with G2P alone'}

    # forward-only rate: the same rollout without recording checkpoints
    sim.set_params(params)
    sim.reset()
    sim.forward(T)
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        sim.reset()
        sim.forward(T)
    f1.record(stream)
    torch.cuda.synchronize()
    fwd_ms = f0.elapsed_time(f1) / args.steps
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([fwd_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        fwd_ms = float(t.item())

    # central differences of each scene's loss w.r.t. its free parameters, all
    # scenes perturbed at once (they are independent), against the adjoint.
    # The float atomics of P2G make each rollout's loss vary in its last bits;
    # `loss_noise_rel` is that variation between two identical rollouts, and
    # `fd_noise_rel` what it contributes to a difference quotient at each step.
    grad_check = None
    fp64_in = None
    if not args.no_fd:
        _, dp_adj = grad_eval(params)
        free = [0, 1, 2] if ys else [0, 2]
        names = {0: 'K', 1: 'tau_y', 2: 'n'}

        def scene_losses(p):
            sim.set_params(p)
            sim.reset()
            f = sim.forward(T)
            diff = (f - target)[..., 0::2].double()
            return (diff * diff).sum(dim=(1, 2)) / float(B * T * 2)

        l_a, l_b = scene_losses(params), scene_losses(params)
        noise = (l_a - l_b).abs()
        grad_check = {'method': 'central differences of each scene loss on the GPU, h = h_rel x |param|',
                      'steps': T, 'loss_noise_rel': float((noise / l_a.abs().clamp_min(1e-300)).max()),
                      'note': 'once the fluid reaches the top band, the sticky top of the reference '
                              '(simulation_functions.py:221-224) makes the loss jump in the parameters and the '
                              'quotients drift from the pointwise derivative by ~1e-3 even in FP64; the adjoint '
                              'is checked against the FP64 oracle adjoint instead (tests)'}
        # the same check over the first substeps only, before the fluid can
        # reach the top band (the 64^3 scene first touches it after ~525)
        Ts = min(T, 400)
        if Ts < T:
            fs_t = target[:, :Ts]

            def short_losses(p):
                sim.set_params(p)
                sim.reset()
                f = sim.forward(Ts)
                diff = (f - fs_t)[..., 0::2].double()
                return (diff * diff).sum(dim=(1, 2)) / float(B * Ts * 2)

            sim.set_params(params)
            sim.reset()
            f = sim.forward(Ts, ckpt_every=ckpt, record=True)
            diff = (f - fs_t)[..., 0::2]
            dF = torch.zeros_like(f)
            dF[..., 0::2] = 2.0 * diff / float(B * Ts * 2)
            dp_s = sim.backward(dF)
            fp64_in = (Ts, dp_s[0].double().cpu().numpy(), fs_t[0].double().cpu().numpy(), float(B * Ts * 2), free,
                       names)
            short = {}
            for hr in sorted({args.fd_h, 1e-2}):
                errs = {}
                for i in free:
                    hs = hr * params[:, i].abs().clamp_min(1e-3)
                    pp, pm = params.clone(), params.clone()
                    pp[:, i] += hs
                    pm[:, i] -= hs
                    fd = (short_losses(pp) - short_losses(pm)) / (2.0 * hs.double())
                    errs[names[i]] = float(((dp_s[:, i].double() - fd).abs() / fd.abs().clamp_min(1e-30)).max())
                short['h_rel=%g' % hr] = {'rel_err': errs, 'rel_err_max': max(errs.values())}
            # FP32 rounding differs between the two perturbed rollouts and
            # dominates the h = 1e-3 quotient (~0.5%); FP64 quotients match
            # the adjoint to 1e-6 over this horizon
            grad_check['first_%d_substeps' % Ts] = short
        for hr in sorted({args.fd_h, 1e-2}):
            errs, nse = {}, {}
            for i in free:
                hs = hr * params[:, i].abs().clamp_min(1e-3)
                pp, pm = params.clone(), params.clone()
                pp[:, i] += hs
                pm[:, i] -= hs
                fd = (scene_losses(pp) - scene_losses(pm)) / (2.0 * hs.double())
                ad = dp_adj[:, i].double()
                errs[names[i]] = float(((ad - fd).abs() / fd.abs().clamp_min(1e-30)).max())
                nse[names[i]] = float((noise / (2.0 * hs.double()) / fd.abs().clamp_min(1e-30)).max())
            grad_check['h_rel=%g' % hr] = {'rel_err': errs, 'rel_err_max': max(errs.values()), 'fd_noise_rel': nse}

    # plain comparison: one scene of the workload alone, per-particle scalar
    # atomics, particles in generation order, no graph
    plain = None
    if not args.no_plain:
        plain = plain_leg([sc], target[:1].contiguous(), params[:1].contiguous(), T, ckpt, args.plain_evals, stream)

    # e2e through the public API with pinned host inputs / host results
    e2e = None
    if not args.no_e2e:
        x0_h = torch.from_numpy(np.concatenate([s.x0() for s in scenes], 0)).float().pin_memory()
        p_h = params.cpu().pin_memory()
        tgt_h = target.cpu().pin_memory()
        h2d = x0_h.numel() * 4 + p_h.numel() * 4 + tgt_h.numel() * 4
        d2h = B * 4 * 4 + 4

        def e2e_step():
            x0_d = x0_h.to(dev, non_blocking=True)
            p_d = p_h.to(dev, non_blocking=True)
            t_d = tgt_h.to(dev, non_blocking=True)
            sim.set_params(p_d)
            sim.set_state(x0_d)
            f = sim.forward(T, ckpt_every=ckpt, record=True)
            diff = (f - t_d)[..., 0::2]
            loss = (diff * diff).mean()
            dF = torch.zeros_like(f)
            dF[..., 0::2] = 2.0 * diff / diff.numel()
            dp = sim.backward(dF)
            return float(loss.item()), dp.cpu()

        e2e_step()
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
        if world > 1:
            import torch.distributed as dist
            t = torch.tensor([e2e_ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_ms = float(t.item())
        e2e = {'value': n_total * T / (e2e_ms / 1e3), 'unit': UNIT, 'h2d_bytes_per_step': int(h2d),
               'd2h_bytes_per_step': int(d2h), 'ms_per_step': e2e_ms}

    status_all = int(st) | int(sim.status())
    opts_used = {k: sim.get_option(k) for k in ('p2g', 'graph', 'block', 'gblock', 'brick_scatter', 'brick_gather',
                                                'fuse', 'fuse_adj', 'resort', 'tight', 'box',
                                                'store_grids', 'overlap', 'lsort', 'pdl', 'lstage', 'gprio', 'prefetch', 'persist')}
    scatter_variant, scatter_fused = sim.get_option('p2g'), sim.get_option('fuse')
    sim.close()
    del sim
    torch.cuda.empty_cache()

    # the batched workload: many scenes per handle against the plain rollout
    batched = None
    if not args.no_batched and args.config != args.batched_config:
        try:
            batched = batched_leg(args, rank, world, dev, stream)
        except Exception as exc:  # reported in the line; the headline stands
            batched = {'error': '%s: %s' % (type(exc).__name__, exc)}
            torch.cuda.empty_cache()

    if rank != 0:
        return 0

    # roofline of the dominant kernel (by total time inside the timed region)
    G = sum(s.desc.n_grid ** 3 for s in scenes)
    NL = sum(s.desc.n_liquid for s in scenes)
    both = {k: (prof[k][0] + (prof[RC[k]][0] if k in RC else 0.0), prof[k][1] + (prof[RC[k]][1] if k in RC else 0))
            for k in KERNEL_BYTES}
    dom = max(KERNEL_BYTES, key=lambda k: both[k][0])
    tot_ms, cnt = both[dom]
    hbm, peak_kind = peaks()
    wl = workload_name(args, scenes, T, ckpt)
    roof = None
    if cnt:  # (the persistent launches of option persist carry no per-kernel split)
        avg_s = tot_ms / 1e3 / cnt
        bp, bn = KERNEL_BYTES[dom]
        alg = bp * NL + bn * G
        achieved = alg / avg_s / 1e9
        roof = {'bound': 'hbm', 'kernel': dom, 'achieved': achieved, 'peak': hbm, 'unit': 'GB/s',
                'frac': achieved / hbm, 'peak_kind': peak_kind, 'alg_bytes_per_launch': alg,
                'avg_launch_us': avg_s * 1e6, 'traffic': ncu_traffic(dom, args.config),
                'launches_per_step': cnt}
    # atomic roofline of the two scatter kernels: vector-RED sectors per launch
    # (committed ncu summary) over the live mean launch time, against the RED
    # sector rate measured on this GPU
    red_roof = None
    if scatter_variant in (1, 4) and not scatter_fused:
        peak_red = red_peak(max(s.desc.n_grid ** 3 for s in scenes))  # one scene's grid: L2-resident
        red_roof = {'unit': 'RED sectors/s', 'peak': peak_red,
                    'peak_kind': 'measured: 32 consecutive float4 nodes per warp RED, L2-resident grid'}
        for k in ('p2g', 'g2p_adj'):
            t_ms, c = both[k]
            if not c:
                continue
            sec = ncu_value('red_sectors_per_launch', k, args.config)
            ach = sec / (t_ms / 1e3 / c) if sec else None
            red_roof[k] = {'sectors_per_launch': sec, 'avg_launch_us': t_ms / c * 1e3, 'achieved': ach,
                           'frac': ach / peak_red if (ach and peak_red) else None}
    # FP32 side of the roofline: the FMA-pipe issue fraction of each particle
    # kernel over its launch (committed ncu summary), beside the FP32 FMA rate
    # measured on this GPU
    fp32_roof = {'peak': fp32_peak(), 'unit': 'flop/s', 'peak_kind': 'measured: independent FMA chains',
                 'fma_pipe_frac': {k: ncu_value('fp32_pipe_frac', k, args.config)
                                   for k in ('p2g', 'grid', 'g2p', 'g2p_adj', 'grid_adj', 'p2g_adj')},
                 'what': 'share of the FMA pipe issue peak used while the kernel runs '
                         '(ncu sm__inst_executed_pipe_fma, of peak sustained active)'}
    # whole-step algorithmic bytes: forward 192 N + 56 G, adjoint 480 N + 112 G per substep
    step_bytes = T * ((192 + 480) * N + (56 + 112) * G)
    kernel_share = {k: round(prof_ovl[k][0] / max(sum(v[0] for v in prof_ovl.values()), 1e-9), 4) for k in KERNELS}
    kernel_us = {'serial': {k: round(prof[k][0] * 1e3 / prof[k][1], 2) for k in KERNELS if prof[k][1]},
                 'overlapped': {k: round(prof_ovl[k][0] * 1e3 / prof_ovl[k][1], 2) for k in KERNELS if prof_ovl[k][1]},
                 'what': 'mean CUDA-event time per launch (us) in one profiled gradient evaluation without graphs: '
                         '"serial" with the reverse pass on one stream (the roofline uses it), "overlapped" with '
                         'the recompute of the next segment on a second stream, as in the timed steps; *_rc = the '
                         'segment recompute'}

    # FP64 oracle check of the gradient (host cores, after all GPU timing)
    if fp64_in is not None and not args.no_fp64:
        Ts, dp0, tgt0, norm, free, names = fp64_in
        Ts_fp = min(args.fp64_substeps, Ts)
        if Ts_fp == Ts:
            try:
                grad_check['fp64'] = fp64_grad_check(sc, params[0].cpu().numpy(), tgt0, Ts, norm, dp0, free, names,
                                                     args.fd_h, os.cpu_count() or 1, K=ckpt)
            except Exception as exc:
                grad_check['fp64'] = {'error': '%s: %s' % (type(exc).__name__, exc)}

    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        Ts = min(args.cpu_sample, T)
        dt = cpu_sample(sc, Ts, threads)
        cpu = {'value': sc.n_particles * Ts / dt, 'unit': UNIT, 'cores': threads, 'kind': 'port',
               'sample': 'oracle FP32 forward + adjoint of the first %d of %d substeps of scene 0 (%d particles)'
                         % (Ts, T, sc.n_particles)}

    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
        'config': {'workload': wl, 'grid': G, 'particles': N, 'substeps': T, 'ckpt_every': ckpt,
                   'scenes_per_gpu': B, 'parallelism': 'scene-sharded (%d scene(s) per GPU)' % B,
                   'l2': 'inputs larger than L2 (checkpoints + segment states ~%.1f GB per step)' %
                         ((T // ckpt + ckpt) * N * 96 / 1e9),
                   'cpu_timings': 'cpu_baseline and the reference arm time the first %d / %d substeps of the %d '
                                  '(forward + adjoint) and report them per particle-substep: a per-substep '
                                  'extrapolation of a prefix, taken before the fluid reaches the walls'
                                  % (min(args.cpu_sample, T), min(args.ref_sample, T), T)},
        'grad_evals_per_s': world * B * 1e3 / ms,
        'forward_value': n_total * T / (fwd_ms / 1e3),
        'kept_grids': kept,
        'grad_check': grad_check,
        'plain': plain,
        'forward_adjoint_roofline_frac': step_bytes / (ms / 1e3) / 1e9 / hbm,
        'roofline': roof,
        'kernel_time_share': kernel_share,
        'kernel_us_per_launch': kernel_us,
        'batched': batched,
        'roofline_l2_red': red_roof,
        'roofline_fp32': fp32_roof,
        'cpu_baseline': cpu,
        'e2e': e2e,
        'gpu_launches': int(launches),
        'options': opts_used,
        'clocks': clk,
        'status_flags': status_all,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == 'reference':
        return run_reference(args)
    return run_ours(args)


if __name__ == '__main__':
    sys.exit(main())
