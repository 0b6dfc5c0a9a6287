// Periodic re-sort of the particle order inside a handle.
//
// The per-particle scatter (P2G, G2P adjoint) sums the contributions of
// neighbouring lanes to shared stencil nodes before its vector atomics, which
// pays off while the lanes of a warp hold particles of consecutive base cells
// of one grid row (the interleaved order the host sets up once).  Particles
// drift between cells as the fluid moves, so the order is rebuilt every K
// substeps (at the checkpoint boundaries of a recorded rollout):
//   resort_count      base cell and rank inside it of every liquid particle
//                     (warp-aggregated counting, as bin_count in binning.cu)
//   launch_scan       cell starts
//   resort_cellorder  liquid particles listed by base cell
//   resort_rows       one CTA per grid row: the new position of each particle
//                     in (row, rank, k) order, inside its scene's liquid range
//   resort_apply      the state and the caller-index map gathered into the new
//                     order
// The reverse pass undoes the permutation on the state adjoint
// (resort_unpermute).  Rod and container particles keep their positions.
// The reference has no counterpart: its particle order never changes.
#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"

namespace dstir {

namespace {

__device__ __forceinline__ int clamp_cell(float v, int n) {
    // fmaxf returns 0 for NaN, so a corrupt position still gets a cell
    return (int)fminf(fmaxf(v, 0.f), (float)(n - 1));
}

__global__ void __launch_bounds__(256) resort_count_kernel(ResortArgs r) {
    __shared__ BlockInfo bi;
    __shared__ float inv_dx;
    __shared__ int n;
    __shared__ long long goff;
    if (threadIdx.x == 0) {
        bi = r.blk[blockIdx.x];
        inv_dx = r.sc[bi.scene].inv_dx;
        n = r.sc[bi.scene].n;
        goff = r.sc[bi.scene].goff;
    }
    __syncthreads();
    long long p = bi.start + threadIdx.x;
    const bool active = p < bi.end;
    if (bi.kind != KIND_LIQUID) {  // block-uniform
        if (active) r.dest[p] = (int)p;
        return;
    }
    long long key = -1;
    if (active) {
        float x0 = r.in[(long long)(OX + 0) * r.stride + p];
        float x1 = r.in[(long long)(OX + 1) * r.stride + p];
        float x2 = r.in[(long long)(OX + 2) * r.stride + p];
        int b0 = clamp_cell(x0 * inv_dx - 0.5f, n), b1 = clamp_cell(x1 * inv_dx - 0.5f, n),
            b2 = clamp_cell(x2 * inv_dx - 0.5f, n);
        key = goff + ((long long)b0 * n + b1) * n + b2;
    }
    const int lane = threadIdx.x & 31;
    unsigned peers = __match_any_sync(0xffffffffu, key);
    int leader = __ffs(peers) - 1;
    int base_rank = 0;
    if (key >= 0 && lane == leader) base_rank = atomicAdd(r.cnt + key, __popc(peers));
    base_rank = __shfl_sync(0xffffffffu, base_rank, leader);
    if (active) {
        r.key[p] = (int)key;
        r.rank[p] = base_rank + __popc(peers & ((1u << lane) - 1u));
    }
}

__global__ void __launch_bounds__(256) resort_cellorder_kernel(ResortArgs r) {
    __shared__ BlockInfo bi;
    if (threadIdx.x == 0) bi = r.blk[blockIdx.x];
    __syncthreads();
    long long p = bi.start + threadIdx.x;
    if (bi.kind != KIND_LIQUID || p >= bi.end) return;
    r.sorted[r.cell_start[r.key[p]] + r.rank[p]] = (int)p;
}

// Block-wide exclusive scan of one int per thread (blockDim.x <= 1024,
// a multiple of 32); returns the exclusive prefix and sets `total`.
__device__ __forceinline__ int block_excl_scan(int v, int& total, int* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int u = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += u;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int y = lane < nw ? sh[lane] : 0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, y, off);
            if (lane >= off) y += u;
        }
        if (lane < nw) sh[lane] = y;
    }
    __syncthreads();
    int excl = x - v + (w > 0 ? sh[w - 1] : 0);
    total = sh[nw - 1];
    __syncthreads();
    return excl;
}

// One CTA per grid row (i, j) of scene blockIdx.y, thread k for cell k.  The
// particles of rank q in the row's cells come before those of rank q+1, each
// group in k order, which puts the particles of rank q of consecutive cells
// into consecutive lanes.
__global__ void __launch_bounds__(1024) resort_rows_kernel(ResortArgs r) {
    __shared__ int sh[32];
    __shared__ int maxc_sh;
    const SceneDev& s = r.sc[blockIdx.y];
    const int n = s.n;
    const long long row = blockIdx.x;
    if (row >= (long long)n * n) return;  // block-uniform
    const int k = threadIdx.x;
    const long long cell0 = s.goff + row * n;
    int c = 0, st0 = 0;
    if (k < n) {
        st0 = r.cell_start[cell0 + k];
        c = r.cell_start[cell0 + k + 1] - st0;
    }
    const long long base_pos = s.p0 + (long long)(r.cell_start[cell0] - r.cell_start[s.goff]);
    if (threadIdx.x == 0) maxc_sh = 0;
    __syncthreads();
    int m = c;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) atomicMax(&maxc_sh, m);
    __syncthreads();
    const int maxc = maxc_sh;
    long long running = 0;
    for (int q = 0; q < maxc; ++q) {
        const int flag = c > q ? 1 : 0;
        int total;
        int excl = block_excl_scan(flag, total, sh);
        if (flag) r.dest[r.sorted[st0 + q]] = (int)(base_pos + running + excl);
        running += total;
    }
}

__global__ void __launch_bounds__(256) resort_apply_kernel(ResortArgs r) {
    __shared__ BlockInfo bi;
    if (threadIdx.x == 0) bi = r.blk[blockIdx.x];
    __syncthreads();
    long long p = bi.start + threadIdx.x;
    if (p >= bi.end) return;
    const long long d = r.dest[p];
#pragma unroll
    for (int c = 0; c < NS; ++c) r.out[(long long)c * r.stride + d] = r.in[(long long)c * r.stride + p];
    r.perm_out[d] = r.perm_in[p];
}

__global__ void __launch_bounds__(256) resort_unpermute_kernel(const float* in, float* out, const int* dest,
                                                               long long stride, long long n) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const long long d = dest[p];
#pragma unroll
    for (int c = 0; c < NS; ++c) out[(long long)c * stride + p] = in[(long long)c * stride + d];
}

}  // namespace

void launch_resort(const ResortArgs& r, int n_blocks, int block, int max_n, int n_scenes, cudaStream_t st) {
    if (n_blocks <= 0) return;
    resort_count_kernel<<<n_blocks, block, 0, st>>>(r);
    launch_scan(r.cnt, r.G + 1, r.bsum, r.cell_start, st);
    resort_cellorder_kernel<<<n_blocks, block, 0, st>>>(r);
    const int row_threads = ((max_n + 31) / 32) * 32;
    resort_rows_kernel<<<dim3((unsigned)((long long)max_n * max_n), (unsigned)n_scenes), row_threads, 0, st>>>(r);
    resort_apply_kernel<<<n_blocks, block, 0, st>>>(r);
}

void launch_unpermute(const float* in, float* out, const int* dest, long long stride, long long n,
                      cudaStream_t st) {
    if (n > 0) resort_unpermute_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, dest, stride, n);
}

}  // namespace dstir
