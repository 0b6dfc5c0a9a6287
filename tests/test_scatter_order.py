"""Host replay of the warp-aggregated scatter's RED traffic for a particle
order (no GPU): the per-block re-interleave that P2G and the G2P adjoint
apply before their scatters (option lsort) must issue fewer 32-byte RED
sectors than the block order once particles have drifted away from the
last re-sort, and no more right after it.

The replay restates three pieces of the CUDA code in numpy:
  - the interleaved order (grid row, rank inside the cell, k) that the
    re-sort builds (resort.cu) and that each block rebuilds
    (local_interleave, device_util.cuh);
  - the run-aggregation emission rule of run_agg_scatter: lane L emits its
    k+0 value, its k+1 value unless lane L+1 has base key+1, and its k+2
    value unless lane L+1 has key+1 or key+2;
  - one 16-byte RED per emitted value; an instruction's lanes that hit the
    same 32-byte sector cost one sector.
Positions come from the FP64 oracle.
"""

import numpy as np

import oracle
from diffstir_gb300 import scene as S


def base_keys(x, n):
    b = np.clip(np.floor(x * n - 0.5).astype(np.int64), 0, n - 1)
    return (b[:, 0] * n + b[:, 1]) * n + b[:, 2]


def interleave(keys, n):
    """Permutation putting `keys` into (row, rank, k) order."""
    o = np.argsort(keys, kind='stable')
    ks = keys[o]
    rank = np.empty(len(keys), np.int64)
    rank[o] = np.arange(len(keys)) - np.searchsorted(ks, ks, side='left')
    return np.lexsort((keys % n, rank, keys // n))


def block_interleave(keys, n, block=256):
    out = np.empty_like(keys)
    for s in range(0, len(keys), block):
        k = keys[s:s + block]
        out[s:s + block] = k[interleave(k, n)]
    return out


def red_sectors(keys, n):
    """RED sectors of one scatter launch, lanes in the order of `keys`."""
    nw = (len(keys) + 31) // 32
    pad = nw * 32 - len(keys)
    kk = np.concatenate([keys, 10**12 + 100 * np.arange(pad)]).reshape(nw, 32)
    act = np.concatenate([np.ones(len(keys), bool), np.zeros(pad, bool)]).reshape(nw, 32)
    d = np.full_like(kk, 99)
    d[:, 1:] = kk[:, 1:] - kk[:, :-1]
    right = np.full_like(kk, 99)            # key difference to lane L+1 when it continues the run
    cont = (d >= 1) & (d <= 2)
    right[:, :-1] = np.where(cont[:, 1:], d[:, 1:], 99)
    emit = [act & (o < right) for o in range(3)]
    total = 0
    for di in range(3):
        for dj in range(3):
            row = kk + (di * n + dj) * n
            for o in range(3):
                sec = np.sort(np.where(emit[o], (row + o) // 2, -1), axis=1)
                total += int(((sec[:, 1:] != sec[:, :-1]) & (sec[:, 1:] >= 0)).sum() + (sec[:, 0] >= 0).sum())
    return total


def test_block_reinterleave_cuts_red_sectors_after_drift():
    n, T0, T1 = 32, 10, 40
    sc = S.small_synthetic_scene(n_grid=n, ppc=8, n_steps=T1, seed=3, lo=(0.2, 0.05, 0.2), hi=(0.8, 0.35, 0.8),
                                 params=(1.0, 0.0, 0.6, 0.0))
    threads = oracle.max_threads()
    x0 = sc.x0()
    _, s0, st = oracle.rollout_last(sc.desc, sc.params, sc.trajectory[:T0 + 1], T0, x0, threads=threads)
    assert st == 0
    _, s1, st = oracle.rollout_last(sc.desc, sc.params, sc.trajectory[T0:T1 + 1], T1 - T0, s0[:, 0:3], s0[:, 3:6],
                                    s0[:, 6:15], s0[:, 15:24], threads=threads)
    assert st == 0
    nl = sc.desc.n_liquid
    order = interleave(base_keys(s0[:nl, 0:3], n), n)   # the re-sort at substep T0
    fresh = base_keys(s0[:nl, 0:3], n)[order]
    drifted = base_keys(s1[:nl, 0:3], n)[order]           # same order, T1 - T0 substeps later
    moved = float(np.mean(fresh != drifted))
    blk_fresh, blk_drift = red_sectors(fresh, n), red_sectors(drifted, n)
    ri_fresh, ri_drift = red_sectors(block_interleave(fresh, n), n), red_sectors(block_interleave(drifted, n), n)
    assert moved > 0.05, moved
    assert blk_drift > 1.1 * blk_fresh, (blk_fresh, blk_drift)
    assert ri_drift < 0.85 * blk_drift, (ri_drift, blk_drift)
    assert ri_fresh <= 1.01 * blk_fresh, (ri_fresh, blk_fresh)


def test_simulator_initial_order_is_the_interleaved_order():
    """The order the Simulator hands the handle (simulator.interleaved_order)
    is the (row, rank, k) order of the re-sort, per scene and particle kind:
    a permutation inside each range, with (i, j, rank, k) non-decreasing."""
    from diffstir_gb300.simulator import interleaved_order
    scenes = [S.small_synthetic_scene(n_grid=16, ppc=4, n_steps=4, seed=21),
              S.small_synthetic_scene(n_grid=20, ppc=8, n_steps=4, seed=22)]
    x0 = np.concatenate([sc.x0() for sc in scenes], 0)
    perm = interleaved_order(scenes, x0)
    off = 0
    for sc in scenes:
        n = sc.desc.n_grid
        for cnt in (sc.desc.n_liquid, sc.desc.n_rod, sc.desc.n_container):
            seg = perm[off:off + cnt]
            assert np.array_equal(np.sort(seg), np.arange(off, off + cnt))
            if cnt:
                keys = base_keys(x0[seg], n)
                # rank of each particle inside its cell, in the order given
                o = np.argsort(keys, kind='stable')
                ks = keys[o]
                rank = np.empty(cnt, np.int64)
                rank[o] = np.arange(cnt) - np.searchsorted(ks, ks, side='left')
                tup = np.stack([keys // n, rank, keys % n], 1)
                assert np.all(np.diff(tup[:, 0]) >= 0)
                same_row = np.diff(tup[:, 0]) == 0
                step = np.diff(tup[:, 1:], axis=0)
                assert np.all((step[same_row, 0] > 0) | ((step[same_row, 0] == 0) & (step[same_row, 1] > 0)))
                assert red_sectors(keys, n) == red_sectors(keys[interleave(keys, n)], n)
            off += cnt
