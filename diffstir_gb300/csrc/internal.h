// Host-side launch interface between the orchestration (api.cu) and the
// kernels (kernels.cu, svd.cu).  Not part of the public C ABI.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace dstir {

struct FwdArgs {
    const SceneDev* sc;
    const BlockInfo* blk;
    const GridBlock* gblk;
    const float* cur;       // state at substep f (SoA, `stride` per component)
    float* next;            // state at substep f+1
    long long stride;
    float4* pm;             // grid momentum (xyz) + mass (w) of this substep
    float4* vo;             // grid velocity after the boundary conditions
    const float* traj;      // [B][traj_len][3]
    int traj_len;
    int f;                  // substep index (trajectory entries f, f+1)
    const float* params;    // [B][4]
    const int* models;      // [B]
    float* force;           // force[s*force_stride + fo*3 + c]
    long long force_stride;
    int fo;
    float* partial;         // [n_blocks][4] per-block partial sums
    unsigned* counters;     // per-scene arrival counters
    unsigned* status;       // DSTIR_STATUS_* word
    int clear_pm;           // grid kernel zeroes pm after reading it
    int batch;
    // fused G2P(f) + P2G(f+1) only: F of state f+2 and the grid of substep f+1
    float* next2 = nullptr;
    float4* pm_next = nullptr;
    // occupied node box of each scene ([B][6]: -imin, -jmin, -kmin, imax, jmax,
    // kmax, all maximised by atomicMax from 0x80808080): the P2G of this
    // substep writes `box`, the fused P2G of the next one `box_next`; the grid
    // update skips nodes outside `box`.  NULL: no box (every node is updated)
    int* box = nullptr;
    int* box_next = nullptr;
    // grid update: blocks [0, n_gblocks) update nodes, the next `batch` blocks
    // compute the rod reaction force of one scene each (set by launch_grid)
    int n_gblocks = 0;
    // warp-aggregated P2G: rebuild the interleaved order inside each block of
    // liquid particles before the scatter
    int lsort = 0;
    // launch with programmatic dependent launch (see pdl_enter)
    int pdl = 0;
    // launch priority of the grid update (a cudaLaunchAttributePriority value;
    // 0: the default).  In the overlapped reverse pass the grid kernels, short
    // and each gating the next kernel of its stream, otherwise wait for SM
    // slots behind the other stream's particle kernels
    int gprio = 0;
    // with lsort: stage the block's state loads and F stores of P2G through
    // shared memory
    int lstage = 0;
};

struct AdjArgs {
    const SceneDev* sc;
    const BlockInfo* blk;
    const GridBlock* gblk;
    const float* cur;        // state at substep f
    long long stride;
    const float4* pm;        // P2G result of substep f
    const float4* vo;        // grid velocity of substep f
    float4* ga;              // adjoint of vo (scatter target, zeroed by the grid adjoint)
    float4* pmb;             // adjoint of pm
    const float* adj_next;   // adjoint of the state at f+1
    float* adj_cur;          // adjoint of the state at f
    const float* traj;
    int traj_len;
    int f;
    const float* params;
    const int* models;
    const float* dforce;     // dL/dforce, same layout as FwdArgs::force
    long long dforce_stride;
    int fo;
    float* pgrad;            // [T][B][4] per-substep parameter gradients
    float* partial;
    unsigned* counters;
    int batch;
    // fused P2G adjoint of substep f with the G2P adjoint of substep f-1 only
    const float* cur2 = nullptr;     // state at substep f-1
    const float4* vo2 = nullptr;     // grid velocity of substep f-1
    float* adj_prev = nullptr;       // adjoint slot of state f-1 (receives its position-adjoint part)
    const int* box = nullptr;        // occupied node box of substep f (see FwdArgs::box) or NULL
    int lsort = 0;                   // warp-aggregated G2P adjoint: see FwdArgs::lsort
    int pdl = 0;                     // see FwdArgs::pdl
    int gprio = 0;                   // launch priority of the grid adjoint (see FwdArgs::gprio)
    // the adjoint kernels' blocks hint L2 to fetch the state that the block
    // pf_dist blocks later reads (0: no hints); n_blocks bounds that index
    int pf_dist = 0;
    int n_blocks = 0;
    int lstage = 0;                  // G2P adjoint: see FwdArgs::lstage
};

// Counting sort of the particles of one substep by stencil-base cell.
struct BinArgs {
    const SceneDev* sc;
    const BlockInfo* blk;
    const float* cur;        // state whose positions are binned
    long long stride;
    int* cnt;                // [G+1] particles per cell (+ overflow bin G); zero on entry, zeroed on exit
    int* key;                // [N] bin of each particle
    int* rank;               // [N] position inside its bin
    int* cell_start;         // [G+2] exclusive prefix of the counts
    int* perm;               // [N] particle indices sorted by bin
    int* bsum;               // scan scratch, bin_scan_blocks(G) entries
    long long G;             // number of bins (the overflow bin is G)
    unsigned* status;
    int key_mode;            // 1: brick-major key (0, the grid node of the stencil base, is unused)
};

// p2g variants: scalar atomics per particle, vector atomics per particle,
// brick tiles in shared memory, vector atomics after warp run aggregation of
// the k-consecutive stencil rows
// (number 2, one thread per binned cell, was retired: slower on every shape)
enum { P2G_PLAIN = 0, P2G_VEC = 1, P2G_BRICK = 3, P2G_WARP = 4 };

// tight: register-cap level of the particle kernels (0, 1 or 2; see kernels.cu)
void launch_p2g(const FwdArgs& a, int n_blocks, int block, int variant, bool svdj, cudaStream_t st, int tight = 0);
void launch_grid(const FwdArgs& a, int n_gblocks, int gblock, cudaStream_t st);
// write_f: G2P also writes F of the next state (see g2p_kernel)
void launch_g2p(const FwdArgs& a, int n_blocks, int block, cudaStream_t st, int tight = 0, bool write_f = false);
// G2P of substep f (into a.next) fused with the stress and P2G scatter of
// substep f+1 (F into a.next2, grid into a.pm_next)
void launch_g2p_p2g(const FwdArgs& a, int n_blocks, int block, int variant, bool svdj, cudaStream_t st,
                    int tight = 0);

void launch_g2p_adj(const AdjArgs& a, int n_blocks, int block, int variant, cudaStream_t st, int tight = 0);
void launch_grid_adj(const AdjArgs& a, int n_gblocks, int gblock, cudaStream_t st);
void launch_p2g_adj(const AdjArgs& a, int n_blocks, int block, bool svdj, cudaStream_t st, int tight = 0);
// P2G adjoint of substep f fused with the G2P adjoint of substep f-1
void launch_p2g_adj_g2p_adj(const AdjArgs& a, int n_blocks, int block, int variant, bool svdj, cudaStream_t st,
                            int tight = 0);

void launch_bin(const BinArgs& b, int n_blocks, int block, cudaStream_t st);
int bin_scan_blocks(long long G);

// scatter mode of the brick kernels: 0 shared tile + atomicAdd, 1 shared tile +
// red.shared, 2 direct global vector atomics in the brick's lane order
void launch_p2g_brick(const FwdArgs& a, const BrickInfo* bricks, int n_bricks, const int* cell_start,
                      const int* perm, long long nbins, bool svdj, int mode, cudaStream_t st);
void launch_g2p_adj_brick(const AdjArgs& a, const BrickInfo* bricks, int n_bricks, const int* cell_start,
                          const int* perm, long long nbins, int mode, cudaStream_t st);
void launch_g2p_brick(const FwdArgs& a, const BrickInfo* bricks, int n_bricks, const int* cell_start,
                      const int* perm, long long nbins, cudaStream_t st);
void launch_p2g_adj_brick(const AdjArgs& a, const BrickInfo* bricks, int n_bricks, const int* cell_start,
                          const int* perm, long long nbins, bool svdj, cudaStream_t st);

void launch_pack_state(const float* x, const float* v, const float* C, const float* F, float* st,
                       long long stride, long long n, cudaStream_t s);
// perm (optional): internal position p goes to caller index perm[p]
void launch_unpack_state(const float* st, long long stride, long long n, float* x, float* v, float* C,
                         float* F, const int* perm, cudaStream_t s);
void launch_iota(int* a, long long n, cudaStream_t s);

// exclusive scan of cnt[0, n) into cell_start[0, n] (cell_start[n] = total);
// zeroes cnt.  bsum: bin_scan_blocks(n - 1) entries.
void launch_scan(int* cnt, long long n, int* bsum, int* cell_start, cudaStream_t st);

// Re-sort of the liquid particles of every scene into the interleaved order
// (stencil-base row (i, j), then rank inside the base cell, then k), so that
// the lanes of a warp hold particles of consecutive base cells of one grid row
// again.  Rod and container particles keep their positions.
struct ResortArgs {
    const SceneDev* sc;
    const BlockInfo* blk;
    const float* in;         // state in the current order
    float* out;              // state in the new order
    long long stride;
    int* cnt;                // [G+1], zero on entry and on exit
    int* cell_start;         // [G+2]
    int* bsum;               // bin_scan_blocks(G) entries
    long long G;             // grid nodes of all scenes
    int* key;                // [N] base cell of each liquid particle
    int* rank;               // [N] rank inside the base cell
    int* sorted;             // [N] liquid particles in base-cell order
    int* dest;               // [N] new position of each particle (identity for rod/container)
    const int* perm_in;      // [N] caller index of each current position
    int* perm_out;           // [N] caller index of each new position
};
void launch_resort(const ResortArgs& r, int n_blocks, int block, int max_n, int n_scenes, cudaStream_t st);
// out[c][p] = in[c][dest[p]]: the adjoint of the re-sort (adjoint in the new
// order -> adjoint in the order before)
void launch_unpermute(const float* in, float* out, const int* dest, long long stride, long long n,
                      cudaStream_t st);
void launch_reduce_pgrad(const float* pgrad, int T, int B, float* out, cudaStream_t s);

// ---------------------------------------------------------------------------
// Persistent segment kernels (option "persist"): one cooperative launch runs
// up to kSegMax substeps of a forward chain, or of a segment's reverse pass,
// with grid-wide barriers between the phases of a substep, instead of one
// launch per phase.  For small scenes, whose substeps are bound by launch
// latency rather than by the GPU's bandwidth.
// ---------------------------------------------------------------------------
constexpr int kSegMax = 50;

// State of the grid barrier, zeroed before every launch.  A block that waits
// longer than the launch's limit sets DSTIR_STATUS_TIMEOUT and `abort`; every
// block then leaves the kernel at its next barrier.
struct GridBar {
    unsigned count;   // arrivals in the current generation
    unsigned gen;     // generation, advanced by the last arrival
    unsigned abort;   // set when a wait ran past the limit
    unsigned pad;
};

struct SegFwdArgs {
    FwdArgs a;                    // fields shared by the substeps; cur, next, pm, vo, box, f, fo set per substep
    const float* cur[kSegMax];    // state read by substep k
    float* next[kSegMax];         // state written by substep k
    float4* pm[kSegMax];
    float4* vo[kSegMax];
    int* box[kSegMax];
    int nsteps;                   // substeps of this launch (<= kSegMax)
    int f0, fo0;                  // substep k uses trajectory index f0 + k and force entry fo0 + k
    int n_pblocks;                // particle blocks (the blk table)
    GridBar* bar;
    long long limit_ns;           // longest wait at a barrier
    int bar_extra;                // arrivals a barrier waits for beyond the grid's blocks (0; tests: 1)
};

struct SegAdjArgs {
    AdjArgs a;                    // fields shared by the substeps; the arrays below set the rest
    const float* cur[kSegMax];    // entry q: the q-th substep of the launch (substeps descending)
    const float4* pm[kSegMax];
    const float4* vo[kSegMax];
    const float* adj_next[kSegMax];
    float* adj_cur[kSegMax];
    const int* box[kSegMax];
    int nsteps;
    int f0, fo0;                  // entry q is substep f0 - q, force entry fo0 - q
    int n_pblocks;
    int n_gblocks;
    GridBar* bar;
    unsigned* status;             // DSTIR_STATUS_* word (the adjoint kernels have none of their own)
    long long limit_ns;
    int bar_extra;
};

// Largest co-resident grid of the persistent kernels (blocks of 256 threads),
// 0 when they cannot be launched cooperatively on this device.
int seg_max_blocks(bool svdj);
cudaError_t launch_seg_fwd(const SegFwdArgs& g, int grid, bool svdj, cudaStream_t st);
cudaError_t launch_seg_adj(const SegAdjArgs& g, int grid, bool svdj, cudaStream_t st);

void launch_svd3(const float* A, float* U, float* S, float* V, long long n, cudaStream_t s);
void launch_svd3_backward(const float* gU, const float* gS, const float* gV, const float* U, const float* S,
                          const float* V, float* gA, long long n, cudaStream_t s);

}  // namespace dstir
