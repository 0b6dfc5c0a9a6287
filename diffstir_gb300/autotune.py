"""Launch-configuration autotuner with a JSON cache.

For a scene shape (grid size, particle count, batch, rod mode, J mode) it times
a short recorded forward + adjoint for each candidate configuration
(P2G variant, particle block size, grid block size, register caps,
per-block re-interleave, CUDA-graph replay) with
CUDA events and keeps the fastest.  Results are cached in a JSON file keyed by
GPU name and scene shape, so a shape is tuned once per machine.

Cache location: ``$DIFFSTIR_AUTOTUNE_CACHE`` or
``~/.cache/diffstir_gb300/autotune.json``.
"""

import json
import os
import time

import numpy as np
import torch

from .simulator import Simulator

CANDIDATES = [
    {'p2g': 4, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 1024, 'graph': 1, 'tight': 1},
    {'p2g': 4, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 256, 'graph': 1, 'tight': 1},
    {'p2g': 4, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 1024, 'graph': 1, 'tight': 2},
    {'p2g': 4, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 256, 'graph': 1, 'tight': 2},
    {'p2g': 4, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 1024, 'graph': 1, 'tight': 3},
    {'p2g': 4, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 256, 'graph': 1, 'tight': 3},
    {'p2g': 4, 'fuse': 1, 'fuse_adj': 1, 'block': 256, 'gblock': 1024, 'graph': 1, 'tight': 1},
    {'p2g': 4, 'fuse': 1, 'fuse_adj': 0, 'block': 256, 'gblock': 1024, 'graph': 1, 'tight': 1},
    {'p2g': 4, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 1024, 'graph': 1, 'tight': 0},
    {'p2g': 4, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 1024, 'graph': 1, 'tight': 1, 'lsort': 0},
    {'p2g': 4, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 1024, 'graph': 1, 'tight': 1, 'pdl': 0},
    {'p2g': 4, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 1024, 'graph': 1, 'tight': 1, 'lstage': 0},
    {'p2g': 4, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 1024, 'graph': 1, 'tight': 1, 'pdl': 2},
    # small scenes fill few SMs with 256-particle blocks
    {'p2g': 4, 'fuse': 0, 'fuse_adj': 0, 'block': 128, 'gblock': 256, 'graph': 1, 'tight': 1},
    {'p2g': 4, 'fuse': 0, 'fuse_adj': 0, 'block': 64, 'gblock': 256, 'graph': 1, 'tight': 1, 'lsort': 0},
    {'p2g': 1, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 1024, 'graph': 1, 'tight': 1},
    {'p2g': 3, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 256, 'graph': 0, 'brick_scatter': 2,
     'brick_gather': 0},
]
# persistent cooperative launches: tried for scenes that fill less than half
# of the GPU's 256-particle block slots at one block per SM, where launch
# latency rather than bandwidth bounds a substep
PERSIST_CANDIDATES = [
    {'p2g': 1, 'fuse': 0, 'fuse_adj': 0, 'block': 256, 'gblock': 256, 'graph': 1, 'tight': 1, 'persist': 1},
]
PERSIST_MAX_PARTICLES = 76 * 256


def cache_path():
    p = os.environ.get('DIFFSTIR_AUTOTUNE_CACHE')
    if p:
        return p
    return os.path.join(os.path.expanduser('~'), '.cache', 'diffstir_gb300', 'autotune.json')


def shape_key(scenes):
    scenes = scenes if isinstance(scenes, (list, tuple)) else [scenes]
    n = max(s.desc.n_grid for s in scenes)
    N = sum(s.n_particles for s in scenes)
    bucket = int(round(np.log2(max(N, 1)) * 2))   # half-octave buckets of the particle count
    rod = scenes[0].desc.rod_mode
    svd = int(any(s.desc.j_mode == 1 for s in scenes))
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else 'cpu'
    return 'v14|%s|n%d|N2^%.1f|B%d|rod%d|svd%d' % (name, n, bucket / 2, len(scenes), rod, svd)


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(cache):
    p = cache_path()
    os.makedirs(os.path.dirname(p), exist_ok=True)
    tmp = p + '.tmp%d' % os.getpid()
    with open(tmp, 'w') as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def time_config(scenes, options, nsteps, ckpt, reps=2):
    """Mean seconds of one recorded forward + adjoint of ``nsteps`` substeps."""
    sim = Simulator(scenes, max_steps=nsteps, options=options)
    B = sim.B
    dF = torch.ones((B, nsteps, 3), device=sim.device) / nsteps

    def once():
        sim.reset()
        sim.forward(nsteps, ckpt_every=ckpt, record=True)
        sim.backward(dF)

    once()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        once()
    e1.record()
    torch.cuda.synchronize()
    sim.close()
    return e0.elapsed_time(e1) / 1e3 / reps


def autotune(scenes, nsteps=200, ckpt=50, candidates=None, use_cache=True, verbose=False):
    """Best options dict for ``scenes`` (a Scene or a list).

    Each candidate times a recorded forward + adjoint of ``nsteps`` substeps.
    The horizon spans several checkpoint segments: the particle order, and
    with it the scatter cost, degrades between re-sorts, so a short run from
    the freshly sorted initial state would favour the wrong kernels."""
    key = shape_key(scenes)
    cache = _load() if use_cache else {}
    if key in cache:
        return dict(cache[key]['options'])
    lst = scenes if isinstance(scenes, (list, tuple)) else [scenes]
    nsteps = max(1, min(nsteps, max(s.n_steps for s in lst)))
    ckpt = min(ckpt, nsteps)
    results = []
    if candidates is None:
        candidates = list(CANDIDATES)
        if sum(s.n_particles for s in lst) <= PERSIST_MAX_PARTICLES:
            candidates += PERSIST_CANDIDATES
    for opt in candidates:
        t0 = time.perf_counter()
        try:
            t = time_config(scenes, opt, nsteps, ckpt)
        except RuntimeError as exc:  # a configuration the handle rejects
            t = float('inf')
            if verbose:
                print('autotune: %s rejected: %s' % (opt, exc))
        results.append((t, opt))
        if verbose:
            print('autotune %-55s %8.3f ms (%.1fs)' % (opt, t * 1e3, time.perf_counter() - t0), flush=True)
    best_t, best = min(results, key=lambda r: r[0])
    cache = _load()
    cache[key] = {'options': best, 'seconds': best_t, 'nsteps': nsteps,
                  'all': [{'options': o, 'seconds': t} for t, o in results]}
    if use_cache:
        _save(cache)
    return dict(best)
