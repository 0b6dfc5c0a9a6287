// Device helpers shared by the particle kernels (kernels.cu) and the binned
// kernels (binning.cu): deterministic block/group reductions, vector atomics,
// SoA state loads, and the liquid stress of P2G (simulation_functions.py:111-152).
#pragma once

#include <cuda_runtime.h>

#include <climits>

#include "common.cuh"
#include "svd.cuh"

namespace dstir {

// ---------------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------------
template <int NV>
__device__ __forceinline__ void block_reduce(float (&v)[NV], float (*sh)[4]) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int c = 0; c < NV; ++c) v[c] += __shfl_down_sync(0xffffffffu, v[c], off);
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < NV; ++c) sh[warp][c] = v[c];
    __syncthreads();
    if (warp == 0) {
        int nw = blockDim.x >> 5;
#pragma unroll
        for (int c = 0; c < NV; ++c) v[c] = lane < nw ? sh[lane][c] : 0.f;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
#pragma unroll
            for (int c = 0; c < NV; ++c) v[c] += __shfl_down_sync(0xffffffffu, v[c], off);
    }
}

// Every block of a (scene, purpose) group publishes its partial sum; the block
// that arrives last adds the partials of the group in block order (so the
// result does not depend on scheduling) and writes it to out[0..NV).  `slot`
// is the block's partial-sum slot (its block index, or its virtual block
// index in a persistent kernel); the group's slots are group_first onwards.
template <int NV>
__device__ __forceinline__ void group_sum(float (&v)[NV], float (*sh)[4], float* partial, unsigned* counter,
                                          int group_first, int group_count, float* out, float scale, int slot) {
    __shared__ bool is_last;
    block_reduce<NV>(v, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) partial[(long long)slot * 4 + c] = v[c];
        __threadfence();
        unsigned prev = atomicAdd(counter, 1u);
        is_last = (prev == (unsigned)(group_count - 1));
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    float acc[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) acc[c] = 0.f;
    const volatile float* vp = partial;
    for (int b = threadIdx.x; b < group_count; b += blockDim.x)
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] += vp[(long long)(group_first + b) * 4 + c];
    block_reduce<NV>(acc, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) out[c] = acc[c] * scale;
        *counter = 0u;
    }
}

// Programmatic dependent launch (option "pdl").  The substep kernels are
// launched with programmatic stream serialisation, so a kernel's blocks may
// become resident while the kernel before it in the stream is still running.
// Each of them therefore waits, before its first access to memory that an
// earlier kernel of the stream writes, until the grids it depends on have
// completed and their writes are visible (griddepcontrol.wait; without the
// launch attribute it returns at once), and then lets the next kernel of the
// stream be launched (launch_dependents: that kernel's own wait still holds
// it until this grid has completed).  Every kernel before the previous one
// has completed by the time a kernel starts (the previous one passed its own
// wait before letting it launch), so tables written before the rollout (block
// tables, scenes, trajectories) may be read before the wait; the one-substep
// kernels do so.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ void red_add4(float4* p, float a, float b, float c, float d) {
    atomicAdd(p, make_float4(a, b, c, d));
}

// ---------------------------------------------------------------------------
// warp run aggregation of the 3x3x3 stencil scatter (p2g variant P2G_WARP)
//
// A particle's 27 stencil nodes form 9 rows of three k-consecutive nodes
// (k is the innermost grid index), so with key = local index of the stencil
// base node, row (i, j) of the stencil covers nodes key+o(i,j)+{0,1,2}, with
// the same o(i,j) for every particle of the scene.  In the interleaved
// particle order a warp holds particles of consecutive base cells of one grid
// row, whose rows overlap their neighbours' by two nodes.  When lane L-1 has
// key-1 (flag a1), two shuffle steps sum the overlapping values before the
// vector RED:
//   1. lane L adds lane L-1's k+2 value into its own k+1 value;
//   2. lane L adds lane L-1's k+1 value (as updated by step 1) into its k+0.
// When lane L-1 has key-2 instead (flag g1: one empty cell between them, the
// rows overlap by one node), step 1 adds lane L-1's k+2 value into lane L's
// k+0 value.  A lane whose k+1 and k+2 values were taken by lane L+1 (n1)
// emits only its k+0 value; one whose k+2 value alone was taken (ng1) emits
// k+0 and k+1.  Every value reaches exactly one RED, whatever the keys, so
// the sums are exact for any particle order; only the number of REDs depends
// on it (34 instead of 96 per row for a warp on 32 consecutive base cells).
// Inactive lanes take distinct negative keys and zero values.  All 32 lanes
// must call these.
// ---------------------------------------------------------------------------
struct RunAgg {
    bool a1;    // lane L-1 has key-1: take its k+1 and k+2 values
    bool g1;    // lane L-1 has key-2: take its k+2 value
    bool n1;    // lane L+1 takes this lane's k+1 and k+2 values
    bool ng1;   // lane L+1 takes this lane's k+2 value only
    bool any;   // some lane of the warp aggregates
};

__device__ __forceinline__ int run_agg_inactive_key() { return -(1 << 29) - 4 * (int)(threadIdx.x & 31); }

__device__ __forceinline__ RunAgg run_agg_flags(int key) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int k1 = __shfl_up_sync(full, key, 1);
    RunAgg r;
    r.a1 = lane >= 1 && k1 == key - 1;
    r.g1 = lane >= 1 && k1 == key - 2;
    const int flags = (r.a1 ? 1 : 0) | (r.g1 ? 2 : 0);
    const int nf = __shfl_down_sync(full, flags, 1);
    r.n1 = lane < 31 && (nf & 1);
    r.ng1 = lane < 31 && (nf & 2);
    r.any = __any_sync(full, flags != 0);
    return r;
}

// Aggregates one stencil row (c0, c1, c2 at nodes row+0..2) across the warp
// and issues this lane's REDs.  NW: float components carried (3 or 4; with 3
// the w component is neither shuffled nor accumulated).
template <int NW>
__device__ __forceinline__ void run_agg_scatter(const RunAgg& r, float4* row, float4 c0, float4 c1, float4 c2,
                                                bool active) {
    const unsigned full = 0xffffffffu;
    if (r.any) {
        float t0 = __shfl_up_sync(full, c2.x, 1), t1 = __shfl_up_sync(full, c2.y, 1),
              t2 = __shfl_up_sync(full, c2.z, 1);
        float t3 = NW == 4 ? __shfl_up_sync(full, c2.w, 1) : 0.f;
        if (r.a1) {
            c1.x += t0;
            c1.y += t1;
            c1.z += t2;
            if (NW == 4) c1.w += t3;
        } else if (r.g1) {
            c0.x += t0;
            c0.y += t1;
            c0.z += t2;
            if (NW == 4) c0.w += t3;
        }
        t0 = __shfl_up_sync(full, c1.x, 1);
        t1 = __shfl_up_sync(full, c1.y, 1);
        t2 = __shfl_up_sync(full, c1.z, 1);
        t3 = NW == 4 ? __shfl_up_sync(full, c1.w, 1) : 0.f;
        if (r.a1) {
            c0.x += t0;
            c0.y += t1;
            c0.z += t2;
            if (NW == 4) c0.w += t3;
        }
    }
    if (!active) return;
    if (NW == 3) c0.w = c1.w = c2.w = 0.f;
    atomicAdd(row, c0);
    if (!r.n1) {
        atomicAdd(row + 1, c1);
        if (!r.ng1) atomicAdd(row + 2, c2);
    }
}

// ---------------------------------------------------------------------------
// CTA-local re-interleave (option "lsort")
//
// The run aggregation above relies on the lanes of a warp holding particles
// of consecutive base cells of one grid row, the order the periodic re-sort
// sets up.  As particles cross cell faces between re-sorts that order decays
// and the number of RED sectors of a 64^3 scene grows from 4.4 M right after a
// re-sort to 10.5 M fifty substeps later (CPU replay of the scatter on the
// FP64 trajectory).  Rebuilding the same (row, rank, k) order inside each CTA
// over its own particles, before the scatter, holds it at 4.8 M one substep
// and 6.4 M fifty substeps after the re-sort.  The block's lanes then process
// the block's particles in that order; only which lane handles which particle
// changes, so the sums are the same up to the order of the float additions.
//
//   key   base cell of the particle (clamped into the grid)
//   rank  its index among the block's particles of that cell: a leader per
//         group of equal keys in a warp (__match_any_sync) adds the group's
//         size to the cell's counter in a shared-memory hash table
//   sort  composite (row - lowest row of the block, rank, k, thread) as one
//         32-bit word, bitonic-sorted over the block (in-warp steps through
//         shuffles, the others through shared memory)
// All threads of the block must call it.
// ---------------------------------------------------------------------------
struct LocalOrderSmem {
    union {
        struct {
            int key[512];
            int cnt[512];
        } h;
        unsigned sortbuf[2][256];
    };
    int rowmin;
};

__device__ __forceinline__ unsigned lsort_hash(int key) { return ((unsigned)key * 2654435761u) >> 23; }

// Bitonic sort (ascending) of one distinct 32-bit word per thread over a block
// of N threads; returns this thread's word of the sorted sequence.  Steps of
// stride < 32 exchange through shuffles, the others through shared memory
// (two buffers, one barrier per step).  Fully unrolled for a compile-time N.
template <int N>
__device__ __forceinline__ unsigned block_bitonic_sort(unsigned v, unsigned (*buf)[256]) {
    const unsigned full = 0xffffffffu;
    const int t = threadIdx.x;
    int b = 0;
#pragma unroll
    for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
        for (int st = size >> 1; st > 0; st >>= 1) {
            unsigned o;
            if (st >= 32) {
                buf[b][t] = v;
                __syncthreads();
                o = buf[b][t ^ st];
                b ^= 1;
            } else {
                o = __shfl_xor_sync(full, v, st);
            }
            const bool take_min = ((t & size) == 0) == ((t & st) == 0);
            v = take_min ? min(v, o) : max(v, o);
        }
    }
    return v;
}

// Returns the block-relative particle slot this thread processes; slots
// holding no particle (>= count) sort last.  N == blockDim.x.
template <int N>
__device__ __forceinline__ int local_interleave(const float* cur, long long stride, long long start, int count,
                                                float inv_dx, int n, LocalOrderSmem& sm) {
    const unsigned full = 0xffffffffu;
    const int t = threadIdx.x, lane = t & 31;
#pragma unroll
    for (int i = t; i < 512; i += N) {
        sm.h.key[i] = -1;
        sm.h.cnt[i] = 0;
    }
    if (t == 0) sm.rowmin = INT_MAX;
    const bool valid = t < count;
    int b[3] = {0, 0, 0};
    if (valid) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float X = __ldg(cur + (long long)(OX + c) * stride + start + t) * inv_dx - 0.5f;
            // fmaxf maps NaN to 0, so a corrupt position still gets a cell
            b[c] = (int)fminf(fmaxf(X, 0.f), (float)(n - 1));
        }
    }
    const int row = b[0] * n + b[1];
    const int key = valid ? row * n + b[2] : -1 - lane;  // invalid lanes: distinct, never inserted
    __syncthreads();
    const int wmin = __reduce_min_sync(full, valid ? row : INT_MAX);
    if (lane == 0 && wmin != INT_MAX) atomicMin(&sm.rowmin, wmin);
    const unsigned peers = __match_any_sync(full, key);
    const int leader = __ffs(peers) - 1;
    int base_rank = 0;
    if (valid && lane == leader) {
        unsigned h = lsort_hash(key);
        // at most N distinct keys in 512 >= 2N slots: a free or matching slot
        // is always found within 512 probes
        for (int probe = 0; probe < 512; ++probe, h = (h + 1) & 511u) {
            const int old = atomicCAS(&sm.h.key[h], -1, key);
            if (old == -1 || old == key) {
                base_rank = atomicAdd(&sm.h.cnt[h], __popc(peers));
                break;
            }
        }
    }
    base_rank = __shfl_sync(full, base_rank, leader);
    const int rank = base_rank + __popc(peers & ((1u << lane) - 1u));
    __syncthreads();  // rowmin final; the hash table is dead from here on
    unsigned v;
    if (valid) {
        const unsigned rrel = (unsigned)min(row - sm.rowmin, 510);
        v = (rrel << 23) | ((unsigned)min(rank, 31) << 18) | ((unsigned)b[2] << 8) | (unsigned)t;
    } else {
        v = 0xFFFFFF00u | (unsigned)t;
    }
    v = block_bitonic_sort<N>(v, sm.sortbuf);
    return (int)(v & 0xFFu);
}

// Dispatch on the block size (64, 128 or 256 threads); any other size keeps
// the block order.
__device__ __forceinline__ int local_interleave_any(const float* cur, long long stride, long long start, int count,
                                                    float inv_dx, int n, LocalOrderSmem& sm) {
    switch (blockDim.x) {
        case 256: return local_interleave<256>(cur, stride, start, count, inv_dx, n, sm);
        case 128: return local_interleave<128>(cur, stride, start, count, inv_dx, n, sm);
        case 64: return local_interleave<64>(cur, stride, start, count, inv_dx, n, sm);
        default: return threadIdx.x;
    }
}

// ---------------------------------------------------------------------------
// occupied node box of a scene
//
// box[0..2] = -(lowest stencil node index) per axis, box[3..5] = highest, all
// maximised with atomicMax from the reset value 0x80808080 (INT_MIN-like), so
// one byte memset empties a box.  A node (i, j, k) lies in the box when
// -box[0] <= i <= box[3] and so on.  Block-wide: every thread of the block
// must call box_update; one thread per block issues the atomics, and only for
// bounds that the (possibly stale) current box does not already hold.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void box_update(int* box, const int base[3], bool valid, int (*sh)[6]) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int v[6];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        v[c] = valid ? -base[c] : INT_MIN;
        v[3 + c] = valid ? base[c] + 2 : INT_MIN;
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) v[c] = __reduce_max_sync(full, v[c]);
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < 6; ++c) sh[w][c] = v[c];
    __syncthreads();
    if (threadIdx.x < 6) {
        int m = INT_MIN;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) m = max(m, sh[q][threadIdx.x]);
        if (m != INT_MIN && m > *(volatile int*)(box + threadIdx.x)) atomicMax(box + threadIdx.x, m);
    }
}

// L2 prefetch hint for components [c0, c0 + ncomp) of the particles
// [start, end) (at most 288 of them) of a [comp][stride] array: thread t
// touches line t % 9 of component t / 9, so 9 * ncomp <= blockDim.x threads
// cover it.  Every address lies inside [start, end).
__device__ __forceinline__ void prefetch_state_l2(const float* st, long long stride, long long start,
                                                  long long end, int c0, int ncomp) {
    const int t = threadIdx.x, comp = t / 9, line = t - comp * 9;
    if (comp >= ncomp || end <= start) return;
    const long long p = min(start + 32LL * line, end - 1);
    asm volatile("prefetch.global.L2 [%0];" ::"l"(st + (long long)(c0 + comp) * stride + p));
}

__device__ __forceinline__ bool box_inside(const int* box, int i, int j, int k) {
    return i >= -box[0] && j >= -box[1] && k >= -box[2] && i <= box[3] && j <= box[4] && k <= box[5];
}

// ---------------------------------------------------------------------------
// state loads
//
// Load policy NC.  The one-substep kernels read their inputs through the
// non-coherent read-only path (ld.global.nc), which is valid only for memory
// that no thread writes while the kernel runs.  The persistent segment
// kernels write, in one phase, what later phases read (states, grids,
// adjoints), so they use plain loads (NC false); the acquire side of their
// grid barrier makes the other blocks' writes visible to those.
// ---------------------------------------------------------------------------
template <bool NC, class T>
__device__ __forceinline__ T ldp(const T* p) {
    if constexpr (NC) return __ldg(p);
    else return *p;
}
template <bool NC = true>
__device__ __forceinline__ void load3(const float* st, long long stride, int o, long long p, float* v) {
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = ldp<NC>(st + (long long)(o + c) * stride + p);
}
template <bool NC = true>
__device__ __forceinline__ void load9(const float* st, long long stride, int o, long long p, float* v) {
#pragma unroll
    for (int c = 0; c < 9; ++c) v[c] = ldp<NC>(st + (long long)(o + c) * stride + p);
}
__device__ __forceinline__ void store3(float* st, long long stride, int o, long long p, const float* v) {
#pragma unroll
    for (int c = 0; c < 3; ++c) st[(long long)(o + c) * stride + p] = v[c];
}
__device__ __forceinline__ void store9(float* st, long long stride, int o, long long p, const float* v) {
#pragma unroll
    for (int c = 0; c < 9; ++c) st[(long long)(o + c) * stride + p] = v[c];
}

// Stress and affine momentum of a liquid particle (p2g :111-152).
struct LiquidP2G {
    float Ft[9];
    float A[9];
    float vv[3];
    float J;
};

// SVDJ: the kernel instantiation that may take J from the SVD (scenes with
// DSTIR_J_SVD); the other one never carries the SVD code.
template <bool SVDJ>
__device__ __forceinline__ void liquid_p2g(const SceneDev& s, int model, const float* prm, const float* v,
                                           const float* C, const float* F, LiquidP2G& o) {
    float IC[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) IC[i] = s.dt * C[i] + ((i % 4 == 0) ? 1.f : 0.f);
    matmul3(IC, F, o.Ft);
    if (SVDJ && s.j_mode == DSTIR_J_SVD) {
        float U[9], sg[3], V[9];
        svd3(o.Ft, U, sg, V);
        o.J = sg[0] * sg[1] * sg[2];
    } else {
        o.J = det3(o.Ft);
    }
    float nrm2 = 0.f;
#pragma unroll
    for (int i = 0; i < 9; ++i) nrm2 += C[i] * C[i];
    float gamma = sqrtf(nrm2) + 1e-6f;
    Visc vs = viscosity<false>(model, prm, gamma);
    float pr = (s.bulk / 2.f) * (o.J - (1.f / o.J) - 1.f) * o.J;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            float Dab = 0.5f * (C[a * 3 + b] + C[b * 3 + a]);
            float sig = vs.eta * Dab + ((a == b) ? pr : 0.f);
            o.A[a * 3 + b] = s.alpha * sig + s.m_liq * C[a * 3 + b];
        }
    o.vv[0] = v[0];
    o.vv[1] = v[1] + s.dt * s.gravity;
    o.vv[2] = v[2];
}


}  // namespace dstir
