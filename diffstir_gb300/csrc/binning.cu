// Per-substep particle binning by brick, and the brick-tiled scatter and
// gather kernels (p2g variant 3).
//
// The reference scatters every particle to its 27 stencil nodes with one
// global atomic per node and component (p2g, simulation_functions.py:155-163;
// Taichi's g2p.grad does the transposed scatter).  Here the particles of each
// substep are first counting-sorted by the 4x4x4-cell brick of their stencil
// base (bin_count -> 3-phase scan -> bin_scatter).  One CTA per brick then
// accumulates its particles' contributions in a 6x6x6-node tile in shared
// memory and flushes each touched node with one vector atomic.
//
// Particles whose stencil leaves the grid go to an overflow bin that the
// extra last blocks of each binned kernel handle without scattering.
#include <cuda_runtime.h>

#include "common.cuh"
#include "device_util.cuh"
#include "internal.h"
#include "adjoint.cuh"

namespace dstir {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_PER_THREAD = 16;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_PER_THREAD;
// CTAs after the last brick / grid block that share the overflow bin
constexpr int OVERFLOW_CTAS = 64;

// ---------------------------------------------------------------------------
// counting sort by cell
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) bin_count_kernel(BinArgs b) {
    __shared__ SceneDev s;
    __shared__ BlockInfo bi;
    if (threadIdx.x == 0) {
        bi = b.blk[blockIdx.x];
        s = b.sc[bi.scene];
    }
    __syncthreads();
    long long p = bi.start + threadIdx.x;
    bool active = p < bi.end;
    long long key = -1;
    if (active) {
        float x[3];
        load3(b.cur, b.stride, OX, p, x);
        int base[3];
        float fx[3];
        if (locate(x, s.inv_dx, s.n, base, fx)) {
            key = b.key_mode ? brick_key(s, base[0], base[1], base[2]) : node_index(s, base[0], base[1], base[2]);
        } else {
            key = b.G;  // overflow bin
            atomicOr(b.status, DSTIR_STATUS_OUT_OF_GRID);
        }
    }
    // warp-aggregated increment: lanes with the same key share one atomic
    const int lane = threadIdx.x & 31;
    unsigned peers = __match_any_sync(0xffffffffu, key);
    int leader = __ffs(peers) - 1;
    int base_rank = 0;
    if (key >= 0 && lane == leader) base_rank = atomicAdd(b.cnt + key, __popc(peers));
    base_rank = __shfl_sync(0xffffffffu, base_rank, leader);
    if (active) {
        b.key[p] = (int)key;
        b.rank[p] = base_rank + __popc(peers & ((1u << lane) - 1u));
    }
}

// block sums of cnt[0, n) in chunks of SCAN_CHUNK
__global__ void __launch_bounds__(SCAN_THREADS) scan_reduce_kernel(const int* cnt, long long n, int* bsum) {
    __shared__ int sh[SCAN_THREADS / 32];
    long long base = (long long)blockIdx.x * SCAN_CHUNK;
    int acc = 0;
    for (int i = threadIdx.x; i < SCAN_CHUNK; i += SCAN_THREADS) {
        long long q = base + i;
        if (q < n) acc += cnt[q];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < SCAN_THREADS / 32; ++w) t += sh[w];
        bsum[blockIdx.x] = t;
    }
}

// exclusive scan of bsum[0, nb) in place (one block of 1024 threads)
__global__ void __launch_bounds__(1024) scan_top_kernel(int* bsum, int nb) {
    __shared__ int warp_tot[32];
    const int per = (nb + 1023) / 1024;
    const int t = threadIdx.x;
    int local = 0;
    for (int i = 0; i < per; ++i) {
        int q = t * per + i;
        if (q < nb) local += bsum[q];
    }
    // inclusive warp scan of the per-thread totals
    int lane = t & 31, w = t >> 5;
    int v = local;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int u = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += u;
    }
    if (lane == 31) warp_tot[w] = v;
    __syncthreads();
    if (w == 0) {
        int x = warp_tot[lane];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += u;
        }
        warp_tot[lane] = x;
    }
    __syncthreads();
    int excl = v - local + (w > 0 ? warp_tot[w - 1] : 0);
    for (int i = 0; i < per; ++i) {
        int q = t * per + i;
        if (q < nb) {
            int c = bsum[q];
            bsum[q] = excl;
            excl += c;
        }
    }
}

// cell_start[q] = exclusive prefix of cnt; cnt is zeroed for the next substep;
// cell_start[n] = total
__global__ void __launch_bounds__(SCAN_THREADS) scan_apply_kernel(int* cnt, long long n, const int* bsum,
                                                                  int* cell_start) {
    __shared__ int warp_tot[SCAN_THREADS / 32];
    long long base = (long long)blockIdx.x * SCAN_CHUNK + (long long)threadIdx.x * SCAN_PER_THREAD;
    int vals[SCAN_PER_THREAD];
    int local = 0;
#pragma unroll
    for (int i = 0; i < SCAN_PER_THREAD; ++i) {
        long long q = base + i;
        vals[i] = (q < n) ? cnt[q] : 0;
        local += vals[i];
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int v = local;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int u = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += u;
    }
    if (lane == 31) warp_tot[w] = v;
    __syncthreads();
    if (w == 0) {
        int x = lane < SCAN_THREADS / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += u;
        }
        if (lane < SCAN_THREADS / 32) warp_tot[lane] = x;
    }
    __syncthreads();
    int excl = bsum[blockIdx.x] + v - local + (w > 0 ? warp_tot[w - 1] : 0);
#pragma unroll
    for (int i = 0; i < SCAN_PER_THREAD; ++i) {
        long long q = base + i;
        if (q < n) {
            cell_start[q] = excl;
            cnt[q] = 0;
            excl += vals[i];
            if (q == n - 1) cell_start[n] = excl;
        }
    }
}

__global__ void __launch_bounds__(256) bin_scatter_kernel(BinArgs b) {
    __shared__ BlockInfo bi;
    if (threadIdx.x == 0) bi = b.blk[blockIdx.x];
    __syncthreads();
    long long p = bi.start + threadIdx.x;
    if (p >= bi.end) return;
    int key = b.key[p];
    b.perm[b.cell_start[key] + b.rank[p]] = (int)p;
}

void launch_bin(const BinArgs& b, int n_blocks, int block, cudaStream_t st) {
    if (n_blocks <= 0) return;
    long long n = b.G + 1;  // cells plus the overflow bin
    int nb = (int)((n + SCAN_CHUNK - 1) / SCAN_CHUNK);
    bin_count_kernel<<<n_blocks, block, 0, st>>>(b);
    scan_reduce_kernel<<<nb, SCAN_THREADS, 0, st>>>(b.cnt, n, b.bsum);
    scan_top_kernel<<<1, 1024, 0, st>>>(b.bsum, nb);
    scan_apply_kernel<<<nb, SCAN_THREADS, 0, st>>>(b.cnt, n, b.bsum, b.cell_start);
    bin_scatter_kernel<<<n_blocks, block, 0, st>>>(b);
}

int bin_scan_blocks(long long G) { return (int)((G + 1 + SCAN_CHUNK - 1) / SCAN_CHUNK); }

void launch_scan(int* cnt, long long n, int* bsum, int* cell_start, cudaStream_t st) {
    int nb = (int)((n + SCAN_CHUNK - 1) / SCAN_CHUNK);
    scan_reduce_kernel<<<nb, SCAN_THREADS, 0, st>>>(cnt, n, bsum);
    scan_top_kernel<<<1, 1024, 0, st>>>(bsum, nb);
    scan_apply_kernel<<<nb, SCAN_THREADS, 0, st>>>(cnt, n, bsum, cell_start);
}

// ---------------------------------------------------------------------------
// per-particle pieces of the brick kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ int particle_kind(const SceneDev& s, long long p) {
    long long q = p - s.p0;
    return q < s.n_liquid ? KIND_LIQUID : (q < (long long)s.n_liquid + s.n_rod ? KIND_ROD : KIND_CONTAINER);
}

// Per-particle P2G quantities (p2g :111-153); writes F[f+1].
template <bool SVDJ>
__device__ __forceinline__ void p2g_particle(const FwdArgs& a, const SceneDev& s, const float* prm, int model,
                                             long long p, int kind, float x[3], float& m, float mv[3], float A[9]) {
    float v[3], C[9], F[9];
    load3(a.cur, a.stride, OX, p, x);
    load3(a.cur, a.stride, OV, p, v);
    load9(a.cur, a.stride, OC, p, C);
    load9(a.cur, a.stride, OF, p, F);
    if (kind == KIND_LIQUID) {
        LiquidP2G q;
        liquid_p2g<SVDJ>(s, model, prm, v, C, F, q);
        store9(a.next, a.stride, OF, p, q.Ft);
        m = s.m_liq;
#pragma unroll
        for (int i = 0; i < 9; ++i) A[i] = q.A[i];
#pragma unroll
        for (int c = 0; c < 3; ++c) mv[c] = m * q.vv[c];
    } else {
        store9(a.next, a.stride, OF, p, F);
        m = (kind == KIND_ROD) ? s.m_rod : s.m_cont;
#pragma unroll
        for (int i = 0; i < 9; ++i) A[i] = m * C[i];
#pragma unroll
        for (int c = 0; c < 3; ++c) mv[c] = m * v[c];
    }
}

__device__ __forceinline__ void g2p_adj_particle_inputs(const AdjArgs& a, const SceneDev& s, const float* fb,
                                                        long long p, int kind, float vnb[3], float xb[3],
                                                        float Cb[9]) {
    load9(a.adj_next, a.stride, OC, p, Cb);
    if (kind == KIND_LIQUID) {
        float ax[3], av[3];
        load3(a.adj_next, a.stride, OX, p, ax);
        load3(a.adj_next, a.stride, OV, p, av);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            vnb[c] = av[c] + s.dt * ax[c];
            xb[c] = ax[c];
        }
    } else if (kind == KIND_ROD && s.rod_mode == DSTIR_ROD_PARTICLES) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            vnb[c] = -fb[c] * s.force_scale;
            xb[c] = 0.f;
        }
    } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) vnb[c] = xb[c] = 0.f;
    }
}

// ---------------------------------------------------------------------------
// brick kernels: one CTA per brick of 4x4x4 cells, the brick's 6x6x6 stencil
// nodes accumulated in shared memory and flushed with one vector atomic per
// touched node.  Thread v handles particle j = v / 64 of cell c = v % 64, so
// the 32 lanes of a warp belong to 32 different cells and, for a given stencil
// offset, add into 32 different tile nodes (no same-address conflicts).
// ---------------------------------------------------------------------------
constexpr int TILE = 6;
constexpr int TILE_NODES = TILE * TILE * TILE;


__device__ __forceinline__ int tile_index(int li, int lj, int lk) { return (li * TILE + lj) * TILE + lk; }

// How a brick kernel adds one stencil contribution:
//   SCATTER_ATOM    shared tile, atomicAdd
//   SCATTER_RED     shared tile, no-return red.shared.add.f32
//   SCATTER_GLOBAL  straight to the global grid with one vector atomic per node
//                   (lanes of a warp hit 32 different nodes, so L2 never
//                   serialises same-address updates inside one request)
enum { SCATTER_ATOM = 0, SCATTER_RED = 1, SCATTER_GLOBAL = 2 };

__device__ __forceinline__ void shared_red_add(float* p, float v) {
    unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("red.shared.add.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}

template <int MODE>
__device__ __forceinline__ void tile_add(float* p, float v) {
    if (MODE == SCATTER_RED)
        shared_red_add(p, v);
    else
        atomicAdd(p, v);
}

// shared prologue: brick header, the 65 cell starts, the largest cell count
struct BrickCtx {
    int cs[65];
    int maxcnt;
};

__device__ __forceinline__ bool brick_prologue(const BrickInfo* bricks, const SceneDev* sc, const int* cell_start,
                                               BrickInfo& br, SceneDev& s, BrickCtx& ctx) {
    if (threadIdx.x == 0) {
        br = bricks[blockIdx.x];
        s = sc[br.scene];
        ctx.maxcnt = 0;
    }
    __syncthreads();
    if (threadIdx.x < 65) ctx.cs[threadIdx.x] = cell_start[br.key0 + threadIdx.x];
    __syncthreads();
    if (threadIdx.x < 64) atomicMax(&ctx.maxcnt, ctx.cs[threadIdx.x + 1] - ctx.cs[threadIdx.x]);
    __syncthreads();
    return ctx.cs[0] != ctx.cs[64];
}

template <bool SVDJ, int MODE>
__global__ void __launch_bounds__(256) p2g_brick_kernel(FwdArgs a, const BrickInfo* __restrict__ bricks,
                                                        const int* __restrict__ cell_start,
                                                        const int* __restrict__ perm, int n_bricks,
                                                        long long nbins) {
    __shared__ SceneDev s;
    __shared__ BrickInfo br;
    __shared__ BrickCtx ctx;
    __shared__ float prm[4];
    __shared__ int model;
    __shared__ float tile[4][TILE_NODES];
    if (blockIdx.x >= (unsigned)n_bricks) {
        // overflow bin: particles whose stencil left the grid get F[f+1], no scatter
        int beg = cell_start[nbins], end = cell_start[nbins + 1];
        const unsigned first = blockIdx.x - (unsigned)(gridDim.x - OVERFLOW_CTAS);
        for (int q = beg + first * blockDim.x + threadIdx.x; q < end; q += OVERFLOW_CTAS * blockDim.x) {
            long long p = perm[q];
            int sc_i = 0;
            while (sc_i + 1 < a.batch && a.sc[sc_i + 1].p0 <= p) ++sc_i;
            SceneDev s2 = a.sc[sc_i];
            float pr[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) pr[i] = a.params[sc_i * 4 + i];
            float x[3], m, mv[3], A[9];
            p2g_particle<SVDJ>(a, s2, pr, a.models[sc_i], p, particle_kind(s2, p), x, m, mv, A);
        }
        return;
    }
    if (!brick_prologue(bricks, a.sc, cell_start, br, s, ctx)) return;
    if (threadIdx.x < 4) prm[threadIdx.x] = a.params[br.scene * 4 + threadIdx.x];
    if (threadIdx.x == 0) model = a.models[br.scene];
    for (int i = threadIdx.x; i < 4 * TILE_NODES; i += blockDim.x) (&tile[0][0])[i] = 0.f;
    __syncthreads();
    const int oi = br.bi * 4, oj = br.bj * 4, ok = br.bk * 4;
    const int nv = ctx.maxcnt * 64;
    for (int v = threadIdx.x; v < nv; v += blockDim.x) {
        const int c = v & 63, j = v >> 6;
        const int q = ctx.cs[c] + j;
        if (q >= ctx.cs[c + 1]) continue;
        long long p = perm[q];
        float x[3], m, mv[3], A[9];
        p2g_particle<SVDJ>(a, s, prm, model, p, particle_kind(s, p), x, m, mv, A);
        const int li = c >> 4, lj = (c >> 2) & 3, lk = c & 3;
        float fx[3] = {x[0] * s.inv_dx - (float)(oi + li), x[1] * s.inv_dx - (float)(oj + lj),
                       x[2] * s.inv_dx - (float)(ok + lk)};
        float w[3][3];
        bspline(fx, w);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int jj = 0; jj < 3; ++jj) {
                float wij = w[i][0] * w[jj][1];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    float W = wij * w[k][2];
                    float dp0 = ((float)i - fx[0]) * s.dx, dp1 = ((float)jj - fx[1]) * s.dx,
                          dp2 = ((float)k - fx[2]) * s.dx;
                    const float g0 = W * (mv[0] + (A[0] * dp0 + A[1] * dp1 + A[2] * dp2));
                    const float g1 = W * (mv[1] + (A[3] * dp0 + A[4] * dp1 + A[5] * dp2));
                    const float g2 = W * (mv[2] + (A[6] * dp0 + A[7] * dp1 + A[8] * dp2));
                    if (MODE == SCATTER_GLOBAL) {
                        red_add4(a.pm + node_index(s, oi + li + i, oj + lj + jj, ok + lk + k), g0, g1, g2, W * m);
                    } else {
                        const int t = tile_index(li + i, lj + jj, lk + k);
                        tile_add<MODE>(&tile[0][t], g0);
                        tile_add<MODE>(&tile[1][t], g1);
                        tile_add<MODE>(&tile[2][t], g2);
                        tile_add<MODE>(&tile[3][t], W * m);
                    }
                }
            }
    }
    if (MODE == SCATTER_GLOBAL) return;
    __syncthreads();
    for (int t = threadIdx.x; t < TILE_NODES; t += blockDim.x) {
        float g3 = tile[3][t], g0 = tile[0][t], g1 = tile[1][t], g2 = tile[2][t];
        if (g3 == 0.f && g0 == 0.f && g1 == 0.f && g2 == 0.f) continue;
        const int gi = oi + t / (TILE * TILE), gj = oj + (t / TILE) % TILE, gk = ok + t % TILE;
        if (gi >= s.n || gj >= s.n || gk >= s.n) continue;
        red_add4(a.pm + node_index(s, gi, gj, gk), g0, g1, g2, g3);
    }
}

template <int MODE>
__global__ void __launch_bounds__(256) g2p_adj_brick_kernel(AdjArgs a, const BrickInfo* __restrict__ bricks,
                                                            const int* __restrict__ cell_start,
                                                            const int* __restrict__ perm, int n_bricks,
                                                            long long nbins) {
    __shared__ SceneDev s;
    __shared__ BrickInfo br;
    __shared__ BrickCtx ctx;
    __shared__ float fb[3];
    __shared__ float tile[3][TILE_NODES];
    __shared__ float4 vt[TILE_NODES];
    if (blockIdx.x >= (unsigned)n_bricks) {
        int beg = cell_start[nbins], end = cell_start[nbins + 1];
        const unsigned first = blockIdx.x - (unsigned)(gridDim.x - OVERFLOW_CTAS);
        for (int q = beg + first * blockDim.x + threadIdx.x; q < end; q += OVERFLOW_CTAS * blockDim.x) {
            long long p = perm[q];
            int sc_i = 0;
            while (sc_i + 1 < a.batch && a.sc[sc_i + 1].p0 <= p) ++sc_i;
            if (particle_kind(a.sc[sc_i], p) == KIND_LIQUID) {
                float ax[3];
                load3(a.adj_next, a.stride, OX, p, ax);
                store3(a.adj_cur, a.stride, OX, p, ax);
            }
        }
        return;
    }
    if (!brick_prologue(bricks, a.sc, cell_start, br, s, ctx)) return;
    if (threadIdx.x == 0) {
        const float* d = a.dforce + br.scene * a.dforce_stride + (long long)a.fo * 3;
        for (int c = 0; c < 3; ++c) fb[c] = d[c];
    }
    const int oi = br.bi * 4, oj = br.bj * 4, ok = br.bk * 4;
    for (int t = threadIdx.x; t < TILE_NODES; t += blockDim.x) {
        tile[0][t] = tile[1][t] = tile[2][t] = 0.f;
        const int gi = oi + t / (TILE * TILE), gj = oj + (t / TILE) % TILE, gk = ok + t % TILE;
        vt[t] = (gi < s.n && gj < s.n && gk < s.n) ? __ldg(a.vo + node_index(s, gi, gj, gk))
                                                   : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    const float c4 = 4.f * s.inv_dx;
    const int nv = ctx.maxcnt * 64;
    for (int v = threadIdx.x; v < nv; v += blockDim.x) {
        const int c = v & 63, jv = v >> 6;
        const int q = ctx.cs[c] + jv;
        if (q >= ctx.cs[c + 1]) continue;
        long long p = perm[q];
        const int kind = particle_kind(s, p);
        float x[3], vnb[3], xb[3], Cb[9];
        load3(a.cur, a.stride, OX, p, x);
        g2p_adj_particle_inputs(a, s, fb, p, kind, vnb, xb, Cb);
        const int li = c >> 4, lj = (c >> 2) & 3, lk = c & 3;
        float fx[3] = {x[0] * s.inv_dx - (float)(oi + li), x[1] * s.inv_dx - (float)(oj + lj),
                       x[2] * s.inv_dx - (float)(ok + lk)};
        float w[3][3], dw[3][3];
        bspline_d(fx, w, dw);
        float fxb[3] = {0.f, 0.f, 0.f};
        const bool liquid = kind == KIND_LIQUID;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int t = tile_index(li + i, lj + j, lk + k);
                    float W = w[i][0] * w[j][1] * w[k][2];
                    float d0 = (float)i - fx[0], d1 = (float)j - fx[1], d2 = (float)k - fx[2];
                    float Cd0 = Cb[0] * d0 + Cb[1] * d1 + Cb[2] * d2;
                    float Cd1 = Cb[3] * d0 + Cb[4] * d1 + Cb[5] * d2;
                    float Cd2 = Cb[6] * d0 + Cb[7] * d1 + Cb[8] * d2;
                    if (MODE == SCATTER_GLOBAL) {
                        red_add4(a.ga + node_index(s, oi + li + i, oj + lj + j, ok + lk + k), W * (vnb[0] + c4 * Cd0),
                                 W * (vnb[1] + c4 * Cd1), W * (vnb[2] + c4 * Cd2), 0.f);
                    } else {
                        tile_add<MODE>(&tile[0][t], W * (vnb[0] + c4 * Cd0));
                        tile_add<MODE>(&tile[1][t], W * (vnb[1] + c4 * Cd1));
                        tile_add<MODE>(&tile[2][t], W * (vnb[2] + c4 * Cd2));
                    }
                    if (liquid) {
                        float4 g = vt[t];
                        float Wb = vnb[0] * g.x + vnb[1] * g.y + vnb[2] * g.z +
                                   c4 * (g.x * Cd0 + g.y * Cd1 + g.z * Cd2);
                        fxb[0] -= c4 * W * (Cb[0] * g.x + Cb[3] * g.y + Cb[6] * g.z);
                        fxb[1] -= c4 * W * (Cb[1] * g.x + Cb[4] * g.y + Cb[7] * g.z);
                        fxb[2] -= c4 * W * (Cb[2] * g.x + Cb[5] * g.y + Cb[8] * g.z);
                        fxb[0] += Wb * dw[i][0] * w[j][1] * w[k][2];
                        fxb[1] += Wb * w[i][0] * dw[j][1] * w[k][2];
                        fxb[2] += Wb * w[i][0] * w[j][1] * dw[k][2];
                    }
                }
        if (liquid) {
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) xb[cc] += s.inv_dx * fxb[cc];
            store3(a.adj_cur, a.stride, OX, p, xb);
        }
    }
    if (MODE == SCATTER_GLOBAL) return;
    __syncthreads();
    for (int t = threadIdx.x; t < TILE_NODES; t += blockDim.x) {
        float g0 = tile[0][t], g1 = tile[1][t], g2 = tile[2][t];
        if (g0 == 0.f && g1 == 0.f && g2 == 0.f) continue;
        const int gi = oi + t / (TILE * TILE), gj = oj + (t / TILE) % TILE, gk = ok + t % TILE;
        if (gi >= s.n || gj >= s.n || gk >= s.n) continue;
        red_add4(a.ga + node_index(s, gi, gj, gk), g0, g1, g2, 0.f);
    }
}

// G2P from a shared-memory tile of the brick's 6x6x6 velocity nodes.  Every
// brick CTA of a scene joins the deterministic rod-force reduction
// (particle rod mode), empty bricks included.
__global__ void __launch_bounds__(256) g2p_brick_kernel(FwdArgs a, const BrickInfo* __restrict__ bricks,
                                                        const int* __restrict__ cell_start,
                                                        const int* __restrict__ perm, int n_bricks,
                                                        long long nbins) {
    __shared__ SceneDev s;
    __shared__ BrickInfo br;
    __shared__ BrickCtx ctx;
    __shared__ float sh[32][4];
    __shared__ float tv[3];
    __shared__ float4 vt[TILE_NODES];
    if (blockIdx.x >= (unsigned)n_bricks) {
        // overflow bin: no gather (v and C of the G2P are zero), as g2p_kernel does
        int beg = cell_start[nbins], end = cell_start[nbins + 1];
        const unsigned first = blockIdx.x - (unsigned)(gridDim.x - OVERFLOW_CTAS);
        for (int q = beg + first * blockDim.x + threadIdx.x; q < end; q += OVERFLOW_CTAS * blockDim.x) {
            long long p = perm[q];
            int sc_i = 0;
            while (sc_i + 1 < a.batch && a.sc[sc_i + 1].p0 <= p) ++sc_i;
            const SceneDev& s2 = a.sc[sc_i];
            const int kind = particle_kind(s2, p);
            const float* t0 = a.traj + ((long long)sc_i * a.traj_len + a.f) * 3;
            float x[3], z[9], outv[3], nx[3];
            load3(a.cur, a.stride, OX, p, x);
#pragma unroll
            for (int c = 0; c < 9; ++c) z[c] = 0.f;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float tvc = (t0[3 + c] - t0[c]) / s2.dt;
                outv[c] = (kind == KIND_ROD) ? tvc : 0.f;
                nx[c] = (kind == KIND_ROD) ? x[c] + tvc * s2.dt : x[c];
            }
            store9(a.next, a.stride, OC, p, z);
            store3(a.next, a.stride, OV, p, outv);
            store3(a.next, a.stride, OX, p, nx);
        }
        return;
    }
    brick_prologue(bricks, a.sc, cell_start, br, s, ctx);
    const int oi = br.bi * 4, oj = br.bj * 4, ok = br.bk * 4;
    if (threadIdx.x == 0) {
        const float* t0 = a.traj + ((long long)br.scene * a.traj_len + a.f) * 3;
        for (int c = 0; c < 3; ++c) tv[c] = (t0[3 + c] - t0[c]) / s.dt;
    }
    if (ctx.cs[0] != ctx.cs[64])
        for (int t = threadIdx.x; t < TILE_NODES; t += blockDim.x) {
            const int gi = oi + t / (TILE * TILE), gj = oj + (t / TILE) % TILE, gk = ok + t % TILE;
            vt[t] = (gi < s.n && gj < s.n && gk < s.n) ? __ldg(a.vo + node_index(s, gi, gj, gk))
                                                       : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    __syncthreads();
    float dv[3] = {0.f, 0.f, 0.f};
    bool any_nan = false;
    const int nv = ctx.maxcnt * 64;
    const float c4 = 4.f * s.inv_dx;
    for (int v = threadIdx.x; v < nv; v += blockDim.x) {
        const int c = v & 63, jv = v >> 6;
        const int q = ctx.cs[c] + jv;
        if (q >= ctx.cs[c + 1]) continue;
        long long p = perm[q];
        const int kind = particle_kind(s, p);
        float x[3];
        load3(a.cur, a.stride, OX, p, x);
        const int li = c >> 4, lj = (c >> 2) & 3, lk = c & 3;
        float fx[3] = {x[0] * s.inv_dx - (float)(oi + li), x[1] * s.inv_dx - (float)(oj + lj),
                       x[2] * s.inv_dx - (float)(ok + lk)};
        float w[3][3];
        bspline(fx, w);
        float nv3[3] = {0.f, 0.f, 0.f}, nC[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) nC[i] = 0.f;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    float4 g = vt[tile_index(li + i, lj + j, lk + k)];
                    float W = w[i][0] * w[j][1] * w[k][2];
                    float d0 = (float)i - fx[0], d1 = (float)j - fx[1], d2 = (float)k - fx[2];
                    float wg0 = W * g.x, wg1 = W * g.y, wg2 = W * g.z;
                    nv3[0] += wg0;
                    nv3[1] += wg1;
                    nv3[2] += wg2;
                    nC[0] += wg0 * d0; nC[1] += wg0 * d1; nC[2] += wg0 * d2;
                    nC[3] += wg1 * d0; nC[4] += wg1 * d1; nC[5] += wg1 * d2;
                    nC[6] += wg2 * d0; nC[7] += wg2 * d1; nC[8] += wg2 * d2;
                }
#pragma unroll
        for (int i = 0; i < 9; ++i) nC[i] *= c4;
        store9(a.next, a.stride, OC, p, nC);
        float nx[3], outv[3];
        if (kind == KIND_LIQUID) {
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                outv[cc] = nv3[cc];
                nx[cc] = x[cc] + s.dt * nv3[cc];
            }
            bool fin = isfinite(nx[0]) && isfinite(nx[1]) && isfinite(nx[2]) && isfinite(nv3[0]) &&
                       isfinite(nv3[1]) && isfinite(nv3[2]);
#pragma unroll
            for (int i = 0; i < 9; ++i) fin = fin && isfinite(nC[i]);
            any_nan = any_nan || !fin;
        } else if (kind == KIND_ROD) {
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                dv[cc] += tv[cc] - nv3[cc];
                outv[cc] = tv[cc];
                nx[cc] = x[cc] + tv[cc] * s.dt;
            }
        } else {
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                outv[cc] = 0.f;
                nx[cc] = x[cc];
            }
        }
        store3(a.next, a.stride, OV, p, outv);
        store3(a.next, a.stride, OX, p, nx);
    }
    if (any_nan) atomicOr(a.status, DSTIR_STATUS_NAN);
    if (s.rod_mode == DSTIR_ROD_PARTICLES && s.n_rod > 0) {
        group_sum<3>(dv, sh, a.partial, a.counters + a.batch + br.scene, blockIdx.x - br.idx, br.count,
                     a.force + br.scene * a.force_stride + (long long)a.fo * 3, s.force_scale, blockIdx.x);
    }
}

// P2G adjoint with the brick's P/M adjoint nodes staged in shared memory.
// Every brick CTA joins the deterministic per-scene parameter-gradient
// reduction, empty bricks included.
template <bool SVDJ>
__global__ void __launch_bounds__(256) p2g_adj_brick_kernel(AdjArgs a, const BrickInfo* __restrict__ bricks,
                                                            const int* __restrict__ cell_start,
                                                            const int* __restrict__ perm, int n_bricks,
                                                            long long nbins) {
    __shared__ SceneDev s;
    __shared__ BrickInfo br;
    __shared__ BrickCtx ctx;
    __shared__ float sh[32][4];
    __shared__ float prm[4];
    __shared__ int model;
    __shared__ float4 gt[TILE_NODES];
    if (blockIdx.x >= (unsigned)n_bricks) {
        // overflow bin: no gather; only the stress / F_tmp adjoint of F[f+1]
        int beg = cell_start[nbins], end = cell_start[nbins + 1];
        const unsigned first = blockIdx.x - (unsigned)(gridDim.x - OVERFLOW_CTAS);
        for (int q = beg + first * blockDim.x + threadIdx.x; q < end; q += OVERFLOW_CTAS * blockDim.x) {
            long long p = perm[q];
            int sc_i = 0;
            while (sc_i + 1 < a.batch && a.sc[sc_i + 1].p0 <= p) ++sc_i;
            SceneDev s2 = a.sc[sc_i];
            float pr[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) pr[i] = a.params[sc_i * 4 + i];
            const int kind = particle_kind(s2, p);
            float m, mv[3], A[9], Ab[9], vvb[3] = {0.f, 0.f, 0.f}, fxb[3] = {0.f, 0.f, 0.f}, pg[4] = {0.f, 0.f, 0.f, 0.f};
            p2g_adj_affine<SVDJ>(a.cur, a.stride, s2, pr, a.models[sc_i], p, kind, m, mv, A);
#pragma unroll
            for (int i = 0; i < 9; ++i) Ab[i] = 0.f;
            p2g_adj_finish<SVDJ>(a, s2, pr, a.models[sc_i], p, kind, m, Ab, vvb, fxb, pg);
        }
        return;
    }
    brick_prologue(bricks, a.sc, cell_start, br, s, ctx);
    if (threadIdx.x < 4) prm[threadIdx.x] = a.params[br.scene * 4 + threadIdx.x];
    if (threadIdx.x == 0) model = a.models[br.scene];
    const int oi = br.bi * 4, oj = br.bj * 4, ok = br.bk * 4;
    if (ctx.cs[0] != ctx.cs[64])
        for (int t = threadIdx.x; t < TILE_NODES; t += blockDim.x) {
            const int gi = oi + t / (TILE * TILE), gj = oj + (t / TILE) % TILE, gk = ok + t % TILE;
            gt[t] = (gi < s.n && gj < s.n && gk < s.n) ? __ldg(a.pmb + node_index(s, gi, gj, gk))
                                                       : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    __syncthreads();
    float pg[4] = {0.f, 0.f, 0.f, 0.f};
    const int nv = ctx.maxcnt * 64;
    for (int v = threadIdx.x; v < nv; v += blockDim.x) {
        const int c = v & 63, jv = v >> 6;
        const int q = ctx.cs[c] + jv;
        if (q >= ctx.cs[c + 1]) continue;
        long long p = perm[q];
        const int kind = particle_kind(s, p);
        const bool liquid = kind == KIND_LIQUID;
        float x[3];
        load3(a.cur, a.stride, OX, p, x);
        float m, mv[3], A[9];
        p2g_adj_affine<SVDJ>(a.cur, a.stride, s, prm, model, p, kind, m, mv, A);
        const int li = c >> 4, lj = (c >> 2) & 3, lk = c & 3;
        float fx[3] = {x[0] * s.inv_dx - (float)(oi + li), x[1] * s.inv_dx - (float)(oj + lj),
                       x[2] * s.inv_dx - (float)(ok + lk)};
        float w[3][3], dw[3][3];
        bspline_d(fx, w, dw);
        float Ab[9], vvb[3] = {0.f, 0.f, 0.f}, fxb[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int i = 0; i < 9; ++i) Ab[i] = 0.f;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    float dp[3] = {((float)i - fx[0]) * s.dx, ((float)j - fx[1]) * s.dx, ((float)k - fx[2]) * s.dx};
                    p2g_adj_node(w[i][0] * w[j][1] * w[k][2], dw[i][0] * w[j][1] * w[k][2],
                                 w[i][0] * dw[j][1] * w[k][2], w[i][0] * w[j][1] * dw[k][2], dp,
                                 gt[tile_index(li + i, lj + j, lk + k)], m, mv, A, s.dx, liquid, Ab, vvb, fxb);
                }
        p2g_adj_finish<SVDJ>(a, s, prm, model, p, kind, m, Ab, vvb, fxb, pg);
    }
    group_sum<4>(pg, sh, a.partial, a.counters + 2 * a.batch + br.scene, blockIdx.x - br.idx, br.count,
                 a.pgrad + ((long long)a.fo * a.batch + br.scene) * 4, 1.f, blockIdx.x);
}

void launch_g2p_brick(const FwdArgs& a, const BrickInfo* bricks, int n_bricks, const int* cell_start,
                      const int* perm, long long nbins, cudaStream_t st) {
    if (n_bricks > 0) g2p_brick_kernel<<<n_bricks + OVERFLOW_CTAS, 256, 0, st>>>(a, bricks, cell_start, perm, n_bricks, nbins);
}

void launch_p2g_adj_brick(const AdjArgs& a, const BrickInfo* bricks, int n_bricks, const int* cell_start,
                          const int* perm, long long nbins, bool svdj, cudaStream_t st) {
    if (n_bricks <= 0) return;
    if (svdj)
        p2g_adj_brick_kernel<true><<<n_bricks + OVERFLOW_CTAS, 256, 0, st>>>(a, bricks, cell_start, perm, n_bricks, nbins);
    else
        p2g_adj_brick_kernel<false><<<n_bricks + OVERFLOW_CTAS, 256, 0, st>>>(a, bricks, cell_start, perm, n_bricks, nbins);
}

template <int MODE>
static void p2g_brick_mode(const FwdArgs& a, const BrickInfo* bricks, int n_bricks, const int* cell_start,
                           const int* perm, long long nbins, bool svdj, cudaStream_t st) {
    const int g = n_bricks + OVERFLOW_CTAS;
    if (svdj)
        p2g_brick_kernel<true, MODE><<<g, 256, 0, st>>>(a, bricks, cell_start, perm, n_bricks, nbins);
    else
        p2g_brick_kernel<false, MODE><<<g, 256, 0, st>>>(a, bricks, cell_start, perm, n_bricks, nbins);
}

void launch_p2g_brick(const FwdArgs& a, const BrickInfo* bricks, int n_bricks, const int* cell_start,
                      const int* perm, long long nbins, bool svdj, int mode, cudaStream_t st) {
    if (n_bricks <= 0) return;
    if (mode == SCATTER_RED)
        p2g_brick_mode<SCATTER_RED>(a, bricks, n_bricks, cell_start, perm, nbins, svdj, st);
    else if (mode == SCATTER_GLOBAL)
        p2g_brick_mode<SCATTER_GLOBAL>(a, bricks, n_bricks, cell_start, perm, nbins, svdj, st);
    else
        p2g_brick_mode<SCATTER_ATOM>(a, bricks, n_bricks, cell_start, perm, nbins, svdj, st);
}

void launch_g2p_adj_brick(const AdjArgs& a, const BrickInfo* bricks, int n_bricks, const int* cell_start,
                          const int* perm, long long nbins, int mode, cudaStream_t st) {
    if (n_bricks <= 0) return;
    const int g = n_bricks + OVERFLOW_CTAS;
    if (mode == SCATTER_RED)
        g2p_adj_brick_kernel<SCATTER_RED><<<g, 256, 0, st>>>(a, bricks, cell_start, perm, n_bricks, nbins);
    else if (mode == SCATTER_GLOBAL)
        g2p_adj_brick_kernel<SCATTER_GLOBAL><<<g, 256, 0, st>>>(a, bricks, cell_start, perm, n_bricks, nbins);
    else
        g2p_adj_brick_kernel<SCATTER_ATOM><<<g, 256, 0, st>>>(a, bricks, cell_start, perm, n_bricks, nbins);
}

}  // namespace dstir
