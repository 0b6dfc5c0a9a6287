// C ABI (include/diffstir.h): handle, device memory, substep orchestration,
// checkpointed forward rollout and the segment-recomputing reverse pass.
//
// The reference keeps the whole trajectory ([max_steps, N] fields,
// src/simulator/initialization.py:155-158) so that ti.ad.Tape can replay
// backward(s) (simulation_functions.py:351-365) from stored states.  Here the
// forward keeps only a checkpoint every K substeps; the reverse pass walks the
// segments last to first, recomputes one segment (keeping its K states and K
// P2G grids), then runs the adjoint substeps of that segment in reverse.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.h"

using namespace dstir;

namespace {
// kernel kinds timed by the optional in-library profiler
// (the *_rc kinds are the same kernels inside the reverse pass's segment
// recompute; "p2g" etc. count the forward rollouts only)
enum { K_P2G = 0, K_GRID, K_G2P, K_G2P_ADJ, K_GRID_ADJ, K_P2G_ADJ, K_BIN, K_G2P_P2G, K_P2G_ADJ_G2P_ADJ, K_OTHER,
       K_P2G_RC, K_GRID_RC, K_G2P_RC, K_BIN_RC, K_G2P_P2G_RC, K_SEG_FWD, K_SEG_ADJ, K_SEG_FWD_RC, K_NUM };
const char* const kKernelNames[K_NUM] = {"p2g",     "grid",     "g2p",     "g2p_adj", "grid_adj",
                                         "p2g_adj", "bin",      "g2p_p2g", "p2g_adj_g2p_adj",
                                         "other",   "p2g_rc",   "grid_rc", "g2p_rc",  "bin_rc", "g2p_p2g_rc",
                                         "seg_fwd", "seg_adj",  "seg_fwd_rc"};

// CUDA-event timing of every launch on the launching stream.  Event pairs live
// in a ring; a pair is read back (synchronising on its stop event) when the
// ring wraps or when the totals are queried.
struct Profiler {
    bool on = false;
    std::vector<cudaEvent_t> start, stop;
    std::vector<int> kind;
    size_t head = 0, pending = 0;
    double total_ms[K_NUM] = {0};
    long long count[K_NUM] = {0};

    void reset() {
        drain();
        for (int k = 0; k < K_NUM; ++k) {
            total_ms[k] = 0;
            count[k] = 0;
        }
    }
    void ensure() {
        if (!start.empty()) return;
        const size_t n = 4096;
        start.resize(n);
        stop.resize(n);
        kind.resize(n);
        for (size_t i = 0; i < n; ++i) {
            cudaEventCreate(&start[i]);
            cudaEventCreate(&stop[i]);
        }
    }
    void consume(size_t i) {
        cudaEventSynchronize(stop[i]);
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, start[i], stop[i]) == cudaSuccess) {
            total_ms[kind[i]] += ms;
            count[kind[i]] += 1;
        }
    }
    void drain() {
        size_t n = start.size();
        while (pending > 0) {
            size_t i = (head + n - pending) % n;
            consume(i);
            --pending;
        }
    }
    size_t begin(int k, cudaStream_t st) {
        ensure();
        size_t n = start.size();
        if (pending == n) {
            consume((head + n - pending) % n);
            --pending;
        }
        size_t i = head;
        kind[i] = k;
        cudaEventRecord(start[i], st);
        return i;
    }
    void end(size_t i, cudaStream_t st) {
        cudaEventRecord(stop[i], st);
        head = (head + 1) % start.size();
        ++pending;
    }
    void destroy() {
        for (auto e : start) cudaEventDestroy(e);
        for (auto e : stop) cudaEventDestroy(e);
        start.clear();
        stop.clear();
    }
};
}  // namespace

struct DstirHandle {
    int B = 0;
    int max_steps = 0;
    std::vector<DstirSceneDesc> desc;
    std::vector<SceneDev> sc_h;
    long long N = 0, stride = 0, G = 0;
    int block = 256, gblock = 1024, p2g_variant = P2G_WARP, use_graph = 1;
    int brick_gather = 1;   // with P2G_BRICK: G2P and the P2G adjoint also gather from brick tiles
    int brick_scatter = 1;  // with P2G_BRICK: 0 shared atomics, 1 shared red, 2 direct global atomics
    int fuse = 0;           // per-particle variants: G2P(f) and P2G(f+1) in one kernel (measured 4% slower at 64^3)
    int fuse_adj = 0;       // per-particle variants: P2G adjoint of f and G2P adjoint of f-1 in one kernel
    std::vector<BlockInfo> blk_h;
    std::vector<GridBlock> gblk_h;
    SceneDev* sc = nullptr;
    BlockInfo* blk = nullptr;
    GridBlock* gblk = nullptr;
    int n_blocks = 0, n_gblocks = 0;

    float* work = nullptr;   // 3 state slots (states f, f+1, f+2 of the fused substep)
    float* ckpt = nullptr;
    long long ckpt_slots = 0;
    float* seg = nullptr;
    long long seg_slots = 0;
    float4* pm = nullptr;     // grid slots (P2G result)
    float4* vo = nullptr;     // grid slots (velocity out)
    long long grid_slots = 0;
    float4* ga = nullptr;
    float4* pmb = nullptr;
    float* adj = nullptr;     // 2 adjoint slots
    float* traj = nullptr;
    float* params = nullptr;
    int* models = nullptr;
    float* force_scratch = nullptr;  // [B][max_steps][3]
    float* pgrad = nullptr;          // [max_steps][B][4]
    float* partial = nullptr;
    long long partial_len = 0;
    unsigned* counters = nullptr;
    unsigned* status = nullptr;
    int* box = nullptr;              // [max_steps][B][6] occupied node box of each substep

    // per-substep binning (p2g variant P2G_BRICK); one (cell_start, perm) slot
    // per substep of a segment, so the reverse pass reuses the recompute's bins
    int* cnt = nullptr;         // [G+1]
    int* bkey = nullptr;        // [stride]
    int* brank = nullptr;       // [stride]
    int* bsum = nullptr;        // scan scratch
    int* cell_start = nullptr;  // [bin_slots][G+2]
    int* perm = nullptr;        // [bin_slots][stride]
    long long bin_slots = 0;
    bool any_svd = false;
    // brick-major binning (p2g variant P2G_BRICK)
    long long nbins_brick = 0;  // sum over scenes of 64 * ceil(n/4)^3
    long long nbins_max = 0;    // bins the bin arrays are sized for: max(G, nbins_brick)
    std::vector<BrickInfo> bricks_h;
    BrickInfo* bricks = nullptr;
    int n_bricks = 0;

    // periodic re-sort of the particle order (per-particle variants): every K
    // substeps of a rollout, at the checkpoint boundaries of a recorded one
    int resort = 1;             // option "resort": 0 never
    int tight = 3;              // option "tight": register-cap level of the particle kernels (0..3)
    int use_box = 1;            // option "box": the grid kernels skip nodes outside the occupied box
    int store_grids = 0;        // option "store_grids": a recorded rollout keeps every substep's grids
    int lsort = 1;              // option "lsort": warp-aggregated scatters re-interleave each block's particles
    int pdl = 1;                // option "pdl": programmatic dependent launch, 1 forward rollouts, 2 everywhere
    int lstage = 3;             // option "lstage": re-interleaved blocks stage their state in shared memory (bit 0 P2G, bit 1 G2P adjoint)
    int gprio = 1;              // option "gprio": grid kernels launched at the device's greatest priority
    int pf_dist = 100;          // option "prefetch": adjoint blocks hint L2 for the block this many later
    int prio_hi = 0;            // that priority (cudaDeviceGetStreamPriorityRange at create)
    bool rec_store = false;     // the recorded rollout kept its grids
    // reverse pass: the recompute of segment s-1 runs on rstream while the
    // adjoint of segment s runs on the caller's stream (double-buffered
    // segment states and grids, its own partial-sum buffer)
    int overlap = 1;            // option "overlap"
    // option "persist": forward chains and the reverse pass's segments run as
    // persistent cooperative launches (seg_fwd_kernel / seg_adj_kernel) with
    // bounded grid barriers; "barrier_limit_us" bounds each wait, and
    // "barrier_test" adds an arrival that never comes, so that every wait
    // runs out (tests of the timeout path)
    int persist = 0;
    long long bar_limit_ns = 2000000000LL;
    int bar_extra = 0;
    GridBar* gbar = nullptr;
    int seg_grid_max = -1;      // co-resident blocks of the persistent kernels (-1: not queried)
    cudaStream_t rstream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_r[2] = {nullptr, nullptr}, ev_a[2] = {nullptr, nullptr};
    float* partial2 = nullptr;
    float* fwd_partial = nullptr;  // partial-sum buffer for the forward kernels being enqueued (NULL: partial)
    int max_n = 0;              // largest n_grid of the batch
    int* rs_cnt = nullptr;      // [G+1]
    int* rs_start = nullptr;    // [G+2]
    int* rs_bsum = nullptr;
    int* rs_key = nullptr;      // [stride]
    int* rs_rank = nullptr;     // [stride]
    int* rs_sorted = nullptr;   // [stride]
    int* rs_dest = nullptr;     // [rs_dest_slots][stride]: permutation that made checkpoint slot c
    long long rs_dest_slots = 0;
    int* perm_cur = nullptr;    // [stride] caller index of each internal position
    int* perm_tmp = nullptr;    // [stride]
    int* perm_rec0 = nullptr;   // [stride] perm_cur at the start of the recorded rollout
    bool perm_id = true;        // perm_cur is the identity
    bool rec_perm_id = true;
    bool rec_resort = false;

    Profiler prof;
    long long launches = 0;  // kernel launches issued since the counter was reset

    // CUDA graphs: the whole forward rollout and the whole reverse pass are
    // captured once per shape on a library-owned stream and replayed
    float* fbuf = nullptr;     // [B][max_steps][3] forces of the last forward
    float* dfbuf = nullptr;    // [B][max_steps][3] dL/dforce of the current backward
    float* dpbuf = nullptr;    // [B][4] dL/dparams
    long long epoch = 0;       // bumped on every (re)allocation; part of the graph keys
    bool capturing = false;
    cudaStream_t gstream = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    cudaGraphExec_t fwd_exec = nullptr, bwd_exec = nullptr;
    long long fwd_key[8] = {0}, bwd_key[8] = {0};
    long long fwd_kernels = 0, bwd_kernels = 0;  // kernel launches in one replay of each graph

    int cur = 0;  // work slot holding the current state
    bool in_recompute = false;  // profiler: launches belong to a segment recompute
    bool recorded = false;
    int rec_t0 = 0, rec_n = 0, rec_K = 0;
    std::string err;
};

namespace {

int fail(DstirHandle* h, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (h) h->err = buf;
    return code;
}

#define CUDA_TRY(h, expr)                                                                      \
    do {                                                                                       \
        cudaError_t e_ = (expr);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail((h), DSTIR_ECUDA, "%s failed: %s", #expr, cudaGetErrorString(e_));    \
    } while (0)

template <class T>
int dalloc(DstirHandle* h, T** p, size_t count, const char* what) {
    if (h) ++h->epoch;
    if (*p) cudaFree(*p);
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(h, DSTIR_ENOMEM, "cudaMalloc of %zu bytes for %s failed: %s", count * sizeof(T), what,
                    cudaGetErrorString(e));
    }
    return DSTIR_OK;
}

inline cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

size_t slot_floats(const DstirHandle* h) { return (size_t)NS * (size_t)h->stride; }

int build_tables(DstirHandle* h) {
    h->blk_h.clear();
    h->gblk_h.clear();
    for (int s = 0; s < h->B; ++s) {
        const SceneDev& sd = h->sc_h[s];
        long long starts[3] = {sd.p0, sd.p0 + sd.n_liquid, sd.p0 + sd.n_liquid + sd.n_rod};
        long long counts[3] = {sd.n_liquid, sd.n_rod, sd.n_container};
        for (int kd = 0; kd < 3; ++kd) {
            long long nb = (counts[kd] + h->block - 1) / h->block;
            for (long long b = 0; b < nb; ++b) {
                BlockInfo bi;
                bi.scene = s;
                bi.kind = kd;
                bi.idx = (int)b;
                bi.count = (int)nb;
                bi.start = starts[kd] + b * h->block;
                bi.end = std::min(starts[kd] + counts[kd], bi.start + h->block);
                h->blk_h.push_back(bi);
            }
        }
        long long gn = (long long)sd.n * sd.n * sd.n;
        long long nb = (gn + h->gblock - 1) / h->gblock;
        for (long long b = 0; b < nb; ++b) {
            GridBlock gb;
            gb.scene = s;
            gb.idx = (int)b;
            gb.count = (int)nb;
            gb.pad = 0;
            gb.start = sd.goff + b * h->gblock;
            gb.end = std::min(sd.goff + gn, gb.start + h->gblock);
            h->gblk_h.push_back(gb);
        }
    }
    h->n_blocks = (int)h->blk_h.size();
    h->n_gblocks = (int)h->gblk_h.size();
    int rc;
    if ((rc = dalloc(h, &h->blk, h->blk_h.size(), "block table"))) return rc;
    if ((rc = dalloc(h, &h->gblk, h->gblk_h.size(), "grid block table"))) return rc;
    CUDA_TRY(h, cudaMemcpy(h->blk, h->blk_h.data(), h->blk_h.size() * sizeof(BlockInfo), cudaMemcpyHostToDevice));
    CUDA_TRY(h, cudaMemcpy(h->gblk, h->gblk_h.data(), h->gblk_h.size() * sizeof(GridBlock),
                           cudaMemcpyHostToDevice));
    // partial sums are indexed by the CTA of any reducing kernel: particle
    // blocks, grid blocks, or bricks (+ the overflow CTAs)
    long long pl = std::max<long long>(std::max(std::max(h->n_blocks, h->n_gblocks), h->n_bricks + 64), 1);
    if (pl > h->partial_len) {
        if ((rc = dalloc(h, &h->partial, (size_t)pl * 4, "partial sums"))) return rc;
        h->partial_len = pl;
        if (h->partial2) {  // the reverse pass reallocates its copy at the new size
            cudaFree(h->partial2);
            h->partial2 = nullptr;
        }
    }
    return DSTIR_OK;
}

int ensure_grid_slots(DstirHandle* h, long long n) {
    if (n <= h->grid_slots) return DSTIR_OK;
    int rc;
    if ((rc = dalloc(h, &h->pm, (size_t)(n * h->G), "P2G grids"))) return rc;
    if ((rc = dalloc(h, &h->vo, (size_t)(n * h->G), "velocity grids"))) return rc;
    h->grid_slots = n;
    CUDA_TRY(h, cudaMemset(h->pm, 0, (size_t)(n * h->G) * sizeof(float4)));
    return DSTIR_OK;
}

FwdArgs fwd_args(DstirHandle* h, const float* cur, float* next, float4* pm, float4* vo, int f, float* force,
                 long long force_stride, int fo, int clear_pm) {
    FwdArgs a;
    a.sc = h->sc;
    a.blk = h->blk;
    a.gblk = h->gblk;
    a.cur = cur;
    a.next = next;
    a.stride = h->stride;
    a.pm = pm;
    a.vo = vo;
    a.traj = h->traj;
    a.traj_len = h->max_steps + 1;
    a.f = f;
    a.params = h->params;
    a.models = h->models;
    a.force = force;
    a.force_stride = force_stride;
    a.fo = fo;
    a.partial = h->fwd_partial ? h->fwd_partial : h->partial;
    a.counters = h->counters;
    a.status = h->status;
    a.clear_pm = clear_pm;
    a.batch = h->B;
    a.next2 = nullptr;
    a.pm_next = nullptr;
    a.lsort = h->lsort;
    // level 1: forward rollouts only; level 2: also the reverse pass's recompute
    a.pdl = h->in_recompute ? h->pdl >= 2 : h->pdl >= 1;
    a.lstage = h->lstage;
    a.gprio = h->gprio ? h->prio_hi : 0;
    return a;
}

// Issue one kernel launch, bracketed by profiler events when profiling is on.
template <class Fn>
void timed(DstirHandle* h, int kind, cudaStream_t st, Fn fn) {
    ++h->launches;
    if (!h->prof.on || h->capturing) {
        fn();
        return;
    }
    if (h->in_recompute) {
        if (kind == K_P2G) kind = K_P2G_RC;
        else if (kind == K_GRID) kind = K_GRID_RC;
        else if (kind == K_G2P) kind = K_G2P_RC;
        else if (kind == K_BIN) kind = K_BIN_RC;
        else if (kind == K_G2P_P2G) kind = K_G2P_P2G_RC;
        else if (kind == K_SEG_FWD) kind = K_SEG_FWD_RC;
    }
    size_t i = h->prof.begin(kind, st);
    fn();
    h->prof.end(i, st);
}

int ensure_bin_slots(DstirHandle* h, long long n) {
    if (n <= h->bin_slots) return DSTIR_OK;
    int rc;
    const long long nb = h->nbins_max;
    if (!h->cnt) {
        if ((rc = dalloc(h, &h->cnt, (size_t)(nb + 1), "bin counts"))) return rc;
        CUDA_TRY(h, cudaMemset(h->cnt, 0, (size_t)(nb + 1) * sizeof(int)));
        if ((rc = dalloc(h, &h->bkey, (size_t)h->stride, "bin keys"))) return rc;
        if ((rc = dalloc(h, &h->brank, (size_t)h->stride, "bin ranks"))) return rc;
        if ((rc = dalloc(h, &h->bsum, (size_t)bin_scan_blocks(nb), "scan scratch"))) return rc;
    }
    if ((rc = dalloc(h, &h->cell_start, (size_t)(n * (nb + 2)), "cell starts"))) return rc;
    if ((rc = dalloc(h, &h->perm, (size_t)(n * h->stride), "bin permutation"))) return rc;
    h->bin_slots = n;
    return DSTIR_OK;
}

bool binned(const DstirHandle* h) { return h->p2g_variant == P2G_BRICK; }

// Occupied-box slot of relative substep k (NULL for the binned variants,
// whose scatter kernels do not track the box: their grid update covers every
// node).
int* box_slot(DstirHandle* h, long long k) {
    if (!h->use_box || binned(h) || k < 0 || k >= h->max_steps) return nullptr;
    return h->box + (size_t)k * h->B * 6;
}

void reset_boxes(DstirHandle* h, long long k0, long long n, cudaStream_t st) {
    if (!h->use_box || binned(h) || n <= 0) return;
    cudaMemsetAsync(h->box + (size_t)k0 * h->B * 6, 0x80, (size_t)n * h->B * 6 * sizeof(int), st);
}

int* slot_cell_start(DstirHandle* h, int slot) { return h->cell_start + (size_t)slot * (h->nbins_max + 2); }
int* slot_perm(DstirHandle* h, int slot) { return h->perm + (size_t)slot * h->stride; }

// One forward substep.  With the binned variant (bricks) the particles of
// `a.cur` are counting-sorted into bin slot `bin_slot` first.
void run_substep(DstirHandle* h, const FwdArgs& a, cudaStream_t st, int bin_slot = 0) {
    if (binned(h)) {
        BinArgs b;
        b.sc = h->sc;
        b.blk = h->blk;
        b.cur = a.cur;
        b.stride = h->stride;
        b.cnt = h->cnt;
        b.key = h->bkey;
        b.rank = h->brank;
        b.cell_start = slot_cell_start(h, bin_slot);
        b.perm = slot_perm(h, bin_slot);
        b.bsum = h->bsum;
        b.G = h->nbins_brick;
        b.status = h->status;
        b.key_mode = 1;
        h->launches += 4;
        timed(h, K_BIN, st, [&] { launch_bin(b, h->n_blocks, h->block, st); });
        timed(h, K_P2G, st, [&] {
            launch_p2g_brick(a, h->bricks, h->n_bricks, b.cell_start, b.perm, b.G, h->any_svd, h->brick_scatter, st);
        });
    } else {
        timed(h, K_P2G, st, [&] { launch_p2g(a, h->n_blocks, h->block, h->p2g_variant, h->any_svd, st, h->tight); });
    }
    timed(h, K_GRID, st, [&] { launch_grid(a, h->n_gblocks, h->gblock, st); });
    if (h->p2g_variant == P2G_BRICK && h->brick_gather)
        timed(h, K_G2P, st, [&] {
            launch_g2p_brick(a, h->bricks, h->n_bricks, slot_cell_start(h, bin_slot), slot_perm(h, bin_slot),
                             h->nbins_brick, st);
        });
    else
        timed(h, K_G2P, st, [&] { launch_g2p(a, h->n_blocks, h->block, st, h->tight); });
}

void run_adj_substep(DstirHandle* h, const AdjArgs& a, cudaStream_t st, int bin_slot = 0) {
    if (h->p2g_variant == P2G_BRICK) {
        timed(h, K_G2P_ADJ, st, [&] {
            launch_g2p_adj_brick(a, h->bricks, h->n_bricks, slot_cell_start(h, bin_slot), slot_perm(h, bin_slot),
                                 h->nbins_brick, h->brick_scatter, st);
        });
    } else {
        const int var = h->p2g_variant;  // P2G_PLAIN, P2G_VEC or P2G_WARP here
        timed(h, K_G2P_ADJ, st, [&] { launch_g2p_adj(a, h->n_blocks, h->block, var, st, h->tight); });
    }
    timed(h, K_GRID_ADJ, st, [&] { launch_grid_adj(a, h->n_gblocks, h->gblock, st); });
    if (h->p2g_variant == P2G_BRICK && h->brick_gather)
        timed(h, K_P2G_ADJ, st, [&] {
            launch_p2g_adj_brick(a, h->bricks, h->n_bricks, slot_cell_start(h, bin_slot), slot_perm(h, bin_slot),
                                 h->nbins_brick, h->any_svd, st);
        });
    else
        timed(h, K_P2G_ADJ, st, [&] { launch_p2g_adj(a, h->n_blocks, h->block, h->any_svd, st, h->tight); });
}

}  // namespace

extern "C" {

int dstir_create(const DstirSceneDesc* scenes, int32_t batch, int32_t max_steps, DstirHandle** out) {
    if (!out) return DSTIR_EINVAL;
    *out = nullptr;
    if (!scenes || batch <= 0 || max_steps <= 0) return DSTIR_EINVAL;
    // grid-node and bin keys are 32-bit in the re-sort and the binned
    // variants: the batch's nodes must fit in INT_MAX (checked before anything
    // is built or allocated)
    {
        long long g_all = 0;
        for (int s = 0; s < batch; ++s) {
            const long long n = scenes[s].n_grid;
            if (n >= 4 && n <= 1024) g_all += n * n * n;
            if (g_all > (long long)INT_MAX) return DSTIR_ERANGE;
        }
    }
    DstirHandle* h = new (std::nothrow) DstirHandle();
    if (!h) return DSTIR_ENOMEM;
    h->B = batch;
    h->max_steps = max_steps;
    h->desc.assign(scenes, scenes + batch);
    long long p0 = 0, g0 = 0;
    for (int s = 0; s < batch; ++s) {
        const DstirSceneDesc& d = scenes[s];
        if (d.n_grid < 4 || d.n_grid > 1024 || d.n_liquid < 0 || d.n_rod < 0 || d.n_container < 0 ||
            d.bound < 0 || !(d.dt > 0.f) || d.model < 0 || d.model > 2 || d.rod_mode < 0 || d.rod_mode > 1 ||
            d.j_mode < 0 || d.j_mode > 1) {
            int rc = fail(h, DSTIR_EINVAL, "scene %d: invalid descriptor", s);
            delete h;
            return rc;
        }
        if (d.rod_mode == DSTIR_ROD_CYLINDER && d.n_rod != 0) {
            delete h;
            return DSTIR_EINVAL;
        }
        SceneDev sd;
        memset(&sd, 0, sizeof(sd));
        sd.n = d.n_grid;
        sd.bound = d.bound;
        sd.rod_mode = d.rod_mode;
        sd.j_mode = d.j_mode;
        sd.container_wall = d.container_wall;
        sd.model = d.model;
        sd.n_liquid = d.n_liquid;
        sd.n_rod = d.n_rod;
        sd.n_container = d.n_container;
        sd.p0 = p0;
        sd.goff = g0;
        sd.nbr = (d.n_grid + 3) / 4;
        sd.koff = h->nbins_brick;
        for (int bi = 0; bi < sd.nbr; ++bi)
            for (int bj = 0; bj < sd.nbr; ++bj)
                for (int bk = 0; bk < sd.nbr; ++bk) {
                    BrickInfo b;
                    b.scene = s;
                    b.bi = bi;
                    b.bj = bj;
                    b.bk = bk;
                    b.key0 = sd.koff + (((long long)bi * sd.nbr + bj) * sd.nbr + bk) * 64;
                    b.idx = (int)(((long long)bi * sd.nbr + bj) * sd.nbr + bk);
                    b.count = sd.nbr * sd.nbr * sd.nbr;
                    h->bricks_h.push_back(b);
                }
        h->nbins_brick += 64LL * sd.nbr * sd.nbr * sd.nbr;
        sd.dt = d.dt;
        sd.dx = 1.f / (float)d.n_grid;
        sd.inv_dx = (float)d.n_grid;
        sd.gravity = d.gravity;
        sd.bulk = d.bulk_modulus;
        sd.alpha = (-d.dt * d.liquid_p_vol * 4.f * sd.inv_dx * sd.inv_dx);
        sd.m_liq = d.liquid_p_mass;
        sd.m_rod = d.rod_p_mass;
        sd.m_cont = d.container_p_mass;
        sd.force_scale = d.force_scale;
        sd.ccx = d.container_cx;
        sd.ccz = d.container_cz;
        sd.cr2 = d.container_r * d.container_r;
        sd.rod_r2 = d.rod_radius * d.rod_radius;
        h->sc_h.push_back(sd);
        if (d.j_mode == DSTIR_J_SVD) h->any_svd = true;
        p0 += (long long)d.n_liquid + d.n_rod + d.n_container;
        g0 += (long long)d.n_grid * d.n_grid * d.n_grid;
        h->max_n = std::max(h->max_n, (int)d.n_grid);
    }
    h->N = p0;
    h->stride = std::max<long long>((p0 + 31) / 32 * 32, 32);
    h->G = g0;
    h->nbins_max = std::max(h->G, h->nbins_brick);
    h->n_bricks = (int)h->bricks_h.size();
    int rc = DSTIR_OK;
    {
        int least = 0, greatest = 0;
        if (cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess) h->prio_hi = greatest;
    }
    std::vector<int> models(batch);
    for (int s = 0; s < batch; ++s) models[s] = scenes[s].model;
    if ((rc = dalloc(h, &h->sc, batch, "scene table")) ||
        (rc = dalloc(h, &h->work, 3 * slot_floats(h), "state")) ||
        (rc = dalloc(h, &h->adj, 2 * slot_floats(h), "adjoint state")) ||
        (rc = dalloc(h, &h->ga, (size_t)h->G, "grid adjoint")) ||
        (rc = dalloc(h, &h->pmb, (size_t)h->G, "P2G adjoint")) ||
        (rc = dalloc(h, &h->traj, (size_t)batch * (max_steps + 1) * 3, "trajectory")) ||
        (rc = dalloc(h, &h->params, (size_t)batch * 4, "parameters")) ||
        (rc = dalloc(h, &h->models, (size_t)batch, "models")) ||
        (rc = dalloc(h, &h->force_scratch, (size_t)batch * max_steps * 3, "force scratch")) ||
        (rc = dalloc(h, &h->fbuf, (size_t)batch * max_steps * 3, "forces")) ||
        (rc = dalloc(h, &h->dfbuf, (size_t)batch * max_steps * 3, "force adjoint")) ||
        (rc = dalloc(h, &h->dpbuf, (size_t)batch * 4, "parameter adjoint")) ||
        (rc = dalloc(h, &h->pgrad, (size_t)max_steps * batch * 4, "parameter gradients")) ||
        (rc = dalloc(h, &h->counters, (size_t)3 * batch, "counters")) ||
        (rc = dalloc(h, &h->status, 1, "status")) || (rc = dalloc(h, &h->bricks, h->bricks_h.size(), "bricks")) ||
        (rc = dalloc(h, &h->box, (size_t)max_steps * batch * 6, "occupied boxes")) ||
        (rc = dalloc(h, &h->perm_cur, (size_t)h->stride, "particle order")) ||
        (rc = dalloc(h, &h->perm_tmp, (size_t)h->stride, "particle order")) ||
        (rc = dalloc(h, &h->perm_rec0, (size_t)h->stride, "particle order")) ||
        (rc = ensure_grid_slots(h, 1)) || (rc = build_tables(h))) {
        std::string msg = h->err;
        dstir_destroy(h);
        return rc;
    }
    cudaError_t e = cudaMemcpy(h->sc, h->sc_h.data(), batch * sizeof(SceneDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(h->bricks, h->bricks_h.data(), h->bricks_h.size() * sizeof(BrickInfo), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->models, models.data(), batch * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(h->counters, 0, 3 * batch * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(h->status, 0, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(h->ga, 0, (size_t)h->G * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemset(h->params, 0, (size_t)batch * 4 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(h->traj, 0, (size_t)batch * (max_steps + 1) * 3 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(h->work, 0, 3 * slot_floats(h) * sizeof(float));
    if (e == cudaSuccess) {
        launch_iota(h->perm_cur, h->stride, 0);
        e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) {
        dstir_destroy(h);
        return DSTIR_ECUDA;
    }
    *out = h;
    return DSTIR_OK;
}

void dstir_destroy(DstirHandle* h) {
    if (!h) return;
    h->prof.drain();
    h->prof.destroy();
    if (h->fwd_exec) cudaGraphExecDestroy(h->fwd_exec);
    if (h->bwd_exec) cudaGraphExecDestroy(h->bwd_exec);
    if (h->gstream) {
        cudaStreamSynchronize(h->gstream);
        cudaStreamDestroy(h->gstream);
    }
    if (h->ev_in) cudaEventDestroy(h->ev_in);
    if (h->ev_out) cudaEventDestroy(h->ev_out);
    if (h->rstream) {
        cudaStreamSynchronize(h->rstream);
        cudaStreamDestroy(h->rstream);
    }
    cudaEvent_t evs[] = {h->ev_fork, h->ev_join, h->ev_r[0], h->ev_r[1], h->ev_a[0], h->ev_a[1]};
    for (cudaEvent_t e : evs)
        if (e) cudaEventDestroy(e);
    void* ptrs[] = {h->sc, h->blk, h->gblk, h->work, h->ckpt, h->seg, h->pm, h->vo, h->ga, h->pmb, h->adj,
                    h->traj, h->params, h->models, h->force_scratch, h->pgrad, h->partial, h->counters, h->status,
                    h->cnt, h->bkey, h->brank, h->bsum, h->cell_start, h->perm, h->fbuf, h->dfbuf, h->dpbuf,
                    h->bricks, h->rs_cnt, h->rs_start, h->rs_bsum, h->rs_key, h->rs_rank, h->rs_sorted,
                    h->rs_dest, h->perm_cur, h->perm_tmp, h->perm_rec0, h->box, h->partial2, h->gbar};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete h;
}

const char* dstir_last_error(const DstirHandle* h) { return h ? h->err.c_str() : "null handle"; }

int dstir_num_particles(const DstirHandle* h, int64_t* n_total, int32_t* batch) {
    if (!h) return DSTIR_EINVAL;
    if (n_total) *n_total = h->N;
    if (batch) *batch = h->B;
    return DSTIR_OK;
}

int dstir_set_state(DstirHandle* h, const float* x, const float* v, const float* C, const float* F, void* stream) {
    if (!h) return DSTIR_EINVAL;
    if (!x) return fail(h, DSTIR_EINVAL, "dstir_set_state: x is required");
    h->cur = 0;
    h->recorded = false;
    timed(h, K_OTHER, S(stream), [&] { launch_pack_state(x, v, C, F, h->work, h->stride, h->N, S(stream)); });
    if (!h->perm_id) launch_iota(h->perm_cur, h->stride, S(stream));
    h->perm_id = true;
    CUDA_TRY(h, cudaGetLastError());
    return DSTIR_OK;
}

int dstir_get_state(DstirHandle* h, float* x, float* v, float* C, float* F, void* stream) {
    if (!h) return DSTIR_EINVAL;
    launch_unpack_state(h->work + (size_t)h->cur * slot_floats(h), h->stride, h->N, x, v, C, F,
                        h->perm_id ? nullptr : h->perm_cur, S(stream));
    CUDA_TRY(h, cudaGetLastError());
    return DSTIR_OK;
}

int dstir_set_params(DstirHandle* h, const float* params, const int32_t* models, void* stream) {
    if (!h) return DSTIR_EINVAL;
    if (params)
        CUDA_TRY(h, cudaMemcpyAsync(h->params, params, (size_t)h->B * 4 * sizeof(float), cudaMemcpyDeviceToDevice,
                                    S(stream)));
    if (models)
        CUDA_TRY(h, cudaMemcpyAsync(h->models, models, (size_t)h->B * sizeof(int), cudaMemcpyDeviceToDevice,
                                    S(stream)));
    h->recorded = false;
    return DSTIR_OK;
}

int dstir_set_trajectory(DstirHandle* h, const float* traj, void* stream) {
    if (!h || !traj) return DSTIR_EINVAL;
    CUDA_TRY(h, cudaMemcpyAsync(h->traj, traj, (size_t)h->B * (h->max_steps + 1) * 3 * sizeof(float),
                                cudaMemcpyDeviceToDevice, S(stream)));
    h->recorded = false;
    return DSTIR_OK;
}

}  // extern "C"

namespace {

// Enqueue a forward rollout; forces go to h->fbuf [B][max_steps][3] at fo = k.
// Returns the work slot that holds the final state.
bool fused(const DstirHandle* h) { return h->fuse && !binned(h); }
bool fused_adj(const DstirHandle* h) { return h->fuse_adj && !binned(h); }


// The persistent path: per-particle vector-RED scatter (p2g 1) in 256-thread
// blocks, no fusion, no processing order, no binning.
bool persist_on(const DstirHandle* h) {
    return h->persist && h->p2g_variant == P2G_VEC && h->block == 256 && !h->fuse && !h->fuse_adj && h->gbar &&
           h->seg_grid_max > 0;
}

int seg_grid(const DstirHandle* h) {
    return std::max(1, std::min(h->seg_grid_max, std::max(h->n_blocks, h->n_gblocks + h->B)));
}

// A forward chain as persistent launches of up to kSegMax substeps.  Slots
// that the grid update does not clear (clear_pm 0) are zeroed first.
template <class SlotFn, class GridFn>
void seg_forward(DstirHandle* h, int t0, int nsteps, SlotFn slot, GridFn grids, float* force, long long fstride,
                 int fo0, int clear_pm, int box0, cudaStream_t st) {
    for (int k0 = 0; k0 < nsteps; k0 += kSegMax) {
        const int L = std::min(kSegMax, nsteps - k0);
        SegFwdArgs g;
        memset(&g, 0, sizeof(g));
        for (int k = 0; k < L; ++k) {
            float4 *pm, *vo;
            grids(k0 + k, pm, vo);
            if (!clear_pm) cudaMemsetAsync(pm, 0, (size_t)h->G * sizeof(float4), st);
            g.cur[k] = slot(k0 + k);
            g.next[k] = slot(k0 + k + 1);
            g.pm[k] = pm;
            g.vo[k] = vo;
            g.box[k] = box_slot(h, box0 + k0 + k);
        }
        g.a = fwd_args(h, g.cur[0], g.next[0], g.pm[0], g.vo[0], t0 + k0, force, fstride, fo0 + k0, clear_pm);
        g.a.n_gblocks = h->n_gblocks;
        g.a.pdl = 0;
        g.nsteps = L;
        g.f0 = t0 + k0;
        g.fo0 = fo0 + k0;
        g.n_pblocks = h->n_blocks;
        g.bar = h->gbar;
        g.limit_ns = h->bar_limit_ns;
        g.bar_extra = h->bar_extra;
        // a launch that stopped at a barrier may leave a group counter of the
        // block reductions behind; every launch starts from clear counters
        cudaMemsetAsync(h->gbar, 0, sizeof(GridBar), st);
        cudaMemsetAsync(h->counters, 0, (size_t)3 * h->B * sizeof(unsigned), st);
        timed(h, K_SEG_FWD, st, [&] { launch_seg_fwd(g, seg_grid(h), h->any_svd, st); });
    }
}

// Forward chain of `nsteps` substeps over the state slots slot(0..nsteps).
// With fusion: P2G(0), then per substep k the grid update and G2P(k) fused
// with P2G(k+1); the last substep ends with a plain G2P unless `skip_last_g2p`.
// `per_step_bins`: binned variants keep the bins of substep k in bin slot k
// (the segment recompute, whose bins the reverse pass reuses); otherwise every
// substep bins into slot 0 (a forward rollout owns a single bin slot).
template <class SlotFn, class GridFn>
void chain_forward(DstirHandle* h, int t0, int nsteps, SlotFn slot, GridFn grids, float* force,
                   long long fstride, int fo0, int clear_pm, bool skip_last_g2p, bool per_step_bins,
                   int box0, cudaStream_t st) {
    // box0: occupied-box slot of substep 0 of this chain
    reset_boxes(h, box0, nsteps, st);
    // Without clear_pm every substep scatters into its own P2G grid slot (the
    // segment recompute, whose grids the reverse pass reads); the slot is
    // zeroed right before its scatter so that the zeroed lines are still in L2
    auto zero_slot = [&](int k) {
        if (clear_pm) return;
        float4 *pm, *vo;
        grids(k, pm, vo);
        cudaMemsetAsync(pm, 0, (size_t)h->G * sizeof(float4), st);
    };
    if (!fused(h) && persist_on(h)) {
        seg_forward(h, t0, nsteps, slot, grids, force, fstride, fo0, clear_pm, box0, st);
        return;
    }
    if (!fused(h)) {
        for (int k = 0; k < nsteps; ++k) {
            float4 *pm, *vo;
            grids(k, pm, vo);
            zero_slot(k);
            FwdArgs a = fwd_args(h, slot(k), slot(k + 1), pm, vo, t0 + k, force, fstride, fo0 + k, clear_pm);
            a.box = box_slot(h, box0 + k);
            run_substep(h, a, st, per_step_bins ? k : 0);
        }
        return;
    }
    {
        float4 *pm, *vo;
        grids(0, pm, vo);
        zero_slot(0);
        FwdArgs a = fwd_args(h, slot(0), slot(1), pm, vo, t0, force, fstride, fo0, clear_pm);
        a.box = box_slot(h, box0);
        timed(h, K_P2G, st, [&] { launch_p2g(a, h->n_blocks, h->block, h->p2g_variant, h->any_svd, st, h->tight); });
    }
    for (int k = 0; k < nsteps; ++k) {
        float4 *pm, *vo;
        grids(k, pm, vo);
        FwdArgs a = fwd_args(h, slot(k), slot(k + 1), pm, vo, t0 + k, force, fstride, fo0 + k, clear_pm);
        a.box = box_slot(h, box0 + k);
        timed(h, K_GRID, st, [&] { launch_grid(a, h->n_gblocks, h->gblock, st); });
        if (k + 1 < nsteps) {
            float4 *pmn, *von;
            grids(k + 1, pmn, von);
            zero_slot(k + 1);
            a.next2 = slot(k + 2);
            a.pm_next = pmn;
            a.box_next = box_slot(h, box0 + k + 1);
            timed(h, K_G2P_P2G, st,
                  [&] { launch_g2p_p2g(a, h->n_blocks, h->block, h->p2g_variant, h->any_svd, st, h->tight); });
        } else if (!skip_last_g2p) {
            timed(h, K_G2P, st, [&] { launch_g2p(a, h->n_blocks, h->block, st, h->tight); });
        }
    }
}

bool resort_on(const DstirHandle* h) { return h->resort && !binned(h) && h->max_n <= 1024; }

int ensure_resort(DstirHandle* h, long long dest_slots) {
    int rc;
    if (!h->rs_cnt) {
        if ((rc = dalloc(h, &h->rs_cnt, (size_t)h->G + 1, "re-sort counts"))) return rc;
        CUDA_TRY(h, cudaMemset(h->rs_cnt, 0, ((size_t)h->G + 1) * sizeof(int)));
        if ((rc = dalloc(h, &h->rs_start, (size_t)h->G + 2, "re-sort cell starts")) ||
            (rc = dalloc(h, &h->rs_bsum, (size_t)bin_scan_blocks(h->G), "re-sort scan")) ||
            (rc = dalloc(h, &h->rs_key, (size_t)h->stride, "re-sort keys")) ||
            (rc = dalloc(h, &h->rs_rank, (size_t)h->stride, "re-sort ranks")) ||
            (rc = dalloc(h, &h->rs_sorted, (size_t)h->stride, "re-sort list")))
            return rc;
    }
    if (dest_slots > h->rs_dest_slots) {
        if ((rc = dalloc(h, &h->rs_dest, (size_t)(dest_slots * h->stride), "re-sort permutations"))) return rc;
        h->rs_dest_slots = dest_slots;
    }
    return DSTIR_OK;
}

// Re-sort state `in` into `out` (different slots); dest receives the
// permutation; perm_cur follows the particles.
void enqueue_resort(DstirHandle* h, const float* in, float* out, int* dest, cudaStream_t st) {
    ResortArgs r;
    r.sc = h->sc;
    r.blk = h->blk;
    r.in = in;
    r.out = out;
    r.stride = h->stride;
    r.cnt = h->rs_cnt;
    r.cell_start = h->rs_start;
    r.bsum = h->rs_bsum;
    r.G = h->G;
    r.key = h->rs_key;
    r.rank = h->rs_rank;
    r.sorted = h->rs_sorted;
    r.dest = dest;
    r.perm_in = h->perm_cur;
    r.perm_out = h->perm_tmp;
    h->launches += 6;  // seven kernels; timed() counts one
    timed(h, K_OTHER, st, [&] { launch_resort(r, h->n_blocks, h->block, h->max_n, h->B, st); });
    cudaMemcpyAsync(h->perm_cur, h->perm_tmp, (size_t)h->N * sizeof(int), cudaMemcpyDeviceToDevice, st);
}

// Number of re-sorts in a rollout of nsteps substeps, chunk length K.
long long resort_count(const DstirHandle* h, int nsteps, int K) {
    return resort_on(h) && K > 0 && nsteps > K ? (nsteps - 1) / K : 0;
}

// Work slot that holds the final state of a forward rollout (the same
// arithmetic as enqueue_forward, for replayed graphs).
int forward_final_slot(const DstirHandle* h, int nsteps, int K, bool record) {
    int a = h->cur;
    if (!resort_count(h, nsteps, K)) return (a + nsteps) % 3;
    for (int k0 = 0;;) {
        int L = std::min(K, nsteps - k0);
        int out = (a + L) % 3;
        if (k0 + L >= nsteps) return out;
        a = record ? out : (out + 1) % 3;
        k0 += L;
    }
}

// Enqueue a forward rollout; forces go to h->fbuf [B][max_steps][3] at fo = k.
// The rollout runs in chunks of K substeps.  Chunk c starts from checkpoint
// slot c when recording, else from a work slot; its intermediate states
// rotate over the three work slots.  With the re-sort on, the state at the
// end of every chunk but the last is re-sorted into the next chunk's start
// slot; otherwise the chunks simply continue ((cur + k) % 3).  Returns the
// work slot of the final state.
int enqueue_forward(DstirHandle* h, int t0, int nsteps, int K, bool record, bool store, cudaStream_t st) {
    size_t sf = slot_floats(h);
    float* W[3] = {h->work, h->work + sf, h->work + 2 * sf};
    const int cur = h->cur;
    // store: substep k scatters into grid slot k and keeps it (and its
    // velocity grid) for the reverse pass; otherwise one slot is reused
    const int clear_pm = store ? 0 : 1;
    if (record) {
        cudaMemcpyAsync(h->ckpt, W[cur], sf * sizeof(float), cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(h->perm_rec0, h->perm_cur, (size_t)h->N * sizeof(int), cudaMemcpyDeviceToDevice, st);
    }
    cudaMemsetAsync(h->pm, 0, (size_t)h->G * sizeof(float4), st);
    int gk0 = 0;  // substep of the current chain's first grid slot (store mode)
    auto grids = [&](int k, float4*& pm, float4*& vo) {
        pm = store ? h->pm + (size_t)(gk0 + k) * h->G : h->pm;
        vo = store ? h->vo + (size_t)(gk0 + k) * h->G : h->vo;
    };
    if (!resort_count(h, nsteps, K)) {
        auto slot = [&](int k) -> float* {
            if (record && k % K == 0 && k < nsteps) return h->ckpt + (size_t)(k / K) * sf;
            return W[(cur + k) % 3];
        };
        chain_forward(h, t0, nsteps, slot, grids, h->fbuf, (long long)h->max_steps * 3, 0, clear_pm, false, false, 0,
                      st);
        return (cur + nsteps) % 3;
    }
    int a = cur;
    float* in = record ? h->ckpt : W[cur];
    for (int c = 0, k0 = 0;; ++c) {
        const int L = std::min(K, nsteps - k0);
        auto slot = [&](int j) -> float* { return j == 0 ? in : W[(a + j) % 3]; };
        gk0 = k0;
        chain_forward(h, t0 + k0, L, slot, grids, h->fbuf, (long long)h->max_steps * 3, k0, clear_pm, false, false, k0,
                      st);
        const int out = (a + L) % 3;
        if (k0 + L >= nsteps) return out;
        float* next = record ? h->ckpt + (size_t)(c + 1) * sf : W[(out + 1) % 3];
        int* dest = h->rs_dest + (size_t)(record ? c + 1 : 0) * h->stride;
        enqueue_resort(h, W[out], next, dest, st);
        in = next;
        a = record ? out : (out + 1) % 3;
        k0 += L;
    }
}

// Run `body(stream)` either directly on `st` or as a cached CUDA graph
// replayed on the library stream (ordered after / before `st` by events).
template <class Body>
int run_maybe_graph(DstirHandle* h, cudaStream_t st, cudaGraphExec_t* exec, long long* key, const long long* want,
                    long long* graph_kernels, Body body) {
    if (!h->use_graph) {
        body(st);
        CUDA_TRY(h, cudaGetLastError());
        return DSTIR_OK;
    }
    if (!h->gstream) {
        CUDA_TRY(h, cudaStreamCreateWithFlags(&h->gstream, cudaStreamNonBlocking));
        CUDA_TRY(h, cudaEventCreateWithFlags(&h->ev_in, cudaEventDisableTiming));
        CUDA_TRY(h, cudaEventCreateWithFlags(&h->ev_out, cudaEventDisableTiming));
    }
    bool hit = *exec != nullptr;
    for (int i = 0; i < 8 && hit; ++i) hit = key[i] == want[i];
    if (!hit) {
        if (*exec) cudaGraphExecDestroy(*exec);
        *exec = nullptr;
        cudaGraph_t g = nullptr;
        CUDA_TRY(h, cudaStreamBeginCapture(h->gstream, cudaStreamCaptureModeThreadLocal));
        h->capturing = true;
        const long long before = h->launches;
        body(h->gstream);
        *graph_kernels = h->launches - before;  // kernels per replay; capturing launches none
        h->launches = before;
        h->capturing = false;
        cudaError_t e = cudaStreamEndCapture(h->gstream, &g);
        if (e != cudaSuccess) return fail(h, DSTIR_ECUDA, "graph capture failed: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(exec, g, h->gprio ? cudaGraphInstantiateFlagUseNodePriority : 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            *exec = nullptr;
            return fail(h, DSTIR_ECUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
        }
        for (int i = 0; i < 8; ++i) key[i] = want[i];
    }
    CUDA_TRY(h, cudaEventRecord(h->ev_in, st));
    CUDA_TRY(h, cudaStreamWaitEvent(h->gstream, h->ev_in, 0));
    CUDA_TRY(h, cudaGraphLaunch(*exec, h->gstream));
    h->launches += *graph_kernels;
    CUDA_TRY(h, cudaEventRecord(h->ev_out, h->gstream));
    CUDA_TRY(h, cudaStreamWaitEvent(st, h->ev_out, 0));
    return DSTIR_OK;
}

}  // namespace

extern "C" {

int dstir_forward(DstirHandle* h, int32_t t0, int32_t nsteps, int32_t ckpt_every, int32_t record, float* force_out,
                  void* stream) {
    if (!h) return DSTIR_EINVAL;
    if (t0 < 0 || nsteps < 0 || (long long)t0 + nsteps > h->max_steps)
        return fail(h, DSTIR_EINVAL, "dstir_forward: steps [%d, %d) outside [0, %d)", t0, t0 + nsteps, h->max_steps);
    if (record && ckpt_every <= 0) return fail(h, DSTIR_EINVAL, "dstir_forward: ckpt_every must be > 0");
    cudaStream_t st = S(stream);
    h->recorded = false;
    if (nsteps == 0) return DSTIR_OK;
    // K: checkpoint interval of a recorded rollout, and the re-sort interval
    int K = ckpt_every > 0 ? std::min(ckpt_every, nsteps) : nsteps;
    long long nseg = record ? (nsteps + K - 1) / K : 0;
    int rc;
    if (record && nseg > h->ckpt_slots) {
        if ((rc = dalloc(h, &h->ckpt, (size_t)nseg * slot_floats(h), "checkpoints"))) return rc;
        h->ckpt_slots = nseg;
    }
    if (binned(h) && (rc = ensure_bin_slots(h, 1))) return rc;
    const long long nres = resort_count(h, nsteps, K);
    if (nres && (rc = ensure_resort(h, record ? nseg : 1))) return rc;
    const bool store = record && h->store_grids && !binned(h) && !fused(h);
    if (store && (rc = ensure_grid_slots(h, nsteps))) return rc;
    long long want[8] = {t0, nsteps, K, record, h->cur, h->epoch,
                         h->p2g_variant * 16 + h->fuse + (nres ? 256 : 0) +
                             (store ? (1LL << 40) : 0) + (h->lsort ? (1LL << 41) : 0) + ((long long)h->pdl << 42) +
                             ((long long)h->lstage << 44) + ((long long)h->gprio << 46),
                         h->block * 4096 + h->gblock};
    rc = run_maybe_graph(h, st, &h->fwd_exec, h->fwd_key, want, &h->fwd_kernels,
                         [&](cudaStream_t s2) { enqueue_forward(h, t0, nsteps, K, record != 0, store, s2); });
    if (rc) return rc;
    const bool start_perm_id = h->perm_id;
    h->cur = forward_final_slot(h, nsteps, K, record != 0);  // also when the chain ran as a replayed graph
    if (nres) h->perm_id = false;
    if (force_out)
        CUDA_TRY(h, cudaMemcpy2DAsync(force_out, (size_t)nsteps * 3 * sizeof(float), h->fbuf,
                                      (size_t)h->max_steps * 3 * sizeof(float), (size_t)nsteps * 3 * sizeof(float),
                                      (size_t)h->B, cudaMemcpyDeviceToDevice, st));
    if (record) {
        h->recorded = true;
        h->rec_t0 = t0;
        h->rec_n = nsteps;
        h->rec_K = K;
        h->rec_resort = nres > 0;
        h->rec_perm_id = start_perm_id;
        h->rec_store = store;
    }
    return DSTIR_OK;
}

int dstir_substep(DstirHandle* h, int32_t f, float* force_out, void* stream) {
    if (!h) return DSTIR_EINVAL;
    if (f < 0 || f >= h->max_steps) return fail(h, DSTIR_EINVAL, "dstir_substep: f=%d outside [0,%d)", f, h->max_steps);
    cudaStream_t st = S(stream);
    h->recorded = false;
    int rc;
    if (binned(h) && (rc = ensure_bin_slots(h, 1))) return rc;
    size_t sf = slot_floats(h);
    float* W[3] = {h->work, h->work + sf, h->work + 2 * sf};
    float* force = force_out ? force_out : h->force_scratch;
    long long fstride = force_out ? 3 : (long long)h->max_steps * 3;
    int fo = force_out ? 0 : f;
    FwdArgs a = fwd_args(h, W[h->cur], W[(h->cur + 1) % 3], h->pm, h->vo, f, force, fstride, fo, 1);
    reset_boxes(h, 0, 1, st);
    a.box = box_slot(h, 0);
    run_substep(h, a, st);
    CUDA_TRY(h, cudaGetLastError());
    h->cur = (h->cur + 1) % 3;
    return DSTIR_OK;
}

}  // extern "C"

namespace {

// Enqueue the reverse pass of the recorded rollout.  dL/dforce is read from
// h->dfbuf ([B][max_steps][3], entry fo = substep - t0); dL/dparams goes to
// h->dpbuf.  Returns the adjoint slot holding dL/d(step-0 state).
bool overlap_on(const DstirHandle* h) { return h->overlap && !binned(h) && !persist_on(h); }

int enqueue_backward(DstirHandle* h, cudaStream_t st) {
    const int n = h->rec_n, K = h->rec_K, t0 = h->rec_t0;
    const long long nseg = (n + K - 1) / K;
    size_t sf = slot_floats(h);
    float* A[2] = {h->adj, h->adj + sf};
    cudaMemsetAsync(A[0], 0, sf * sizeof(float), st);  // adjoint of the final state: zero
    cudaMemsetAsync(h->ga, 0, (size_t)h->G * sizeof(float4), st);
    cudaMemsetAsync(h->pgrad, 0, (size_t)n * h->B * 4 * sizeof(float), st);
    const bool ovl = overlap_on(h) && nseg >= 2;
    // buffer b of the segment states (K-1 slots) and grids (K slots); with the
    // overlap, segment sgi uses buffer sgi & 1
    auto buf = [&](long long sgi) -> int { return ovl ? (int)(sgi & 1) : 0; };
    auto seg_slot = [&](long long sgi, int j) -> float* {
        return j == 0 ? h->ckpt + (size_t)sgi * sf : h->seg + ((size_t)buf(sgi) * K + (j - 1)) * sf;
    };
    // grid slot of substep k of segment sgi: the segment's own slots, or the
    // forward's slot s0 + k when the rollout kept its grids
    auto grid_slot = [&](long long sgi, int k) -> size_t {
        return h->rec_store ? (size_t)(sgi * K + k) : (size_t)buf(sgi) * K + k;
    };
    auto recompute = [&](long long sgi, cudaStream_t s) {
        const int s0 = (int)(sgi * K);
        const int L = std::min(K, n - s0);
        auto slot = [&](int j) -> float* { return seg_slot(sgi, j); };
        auto grids = [&](int k, float4*& pm, float4*& vo) {
            pm = h->pm + grid_slot(sgi, k) * h->G;
            vo = h->vo + grid_slot(sgi, k) * h->G;
        };
        h->in_recompute = true;
        if (ovl) h->fwd_partial = h->partial2;
        if (h->rec_store) {
            // states only: G2P from the kept velocity grids, with F of the next
            // state written by G2P since P2G does not run
            for (int k = 0; k + 1 < L; ++k) {
                float4 *pm, *vo;
                grids(k, pm, vo);
                FwdArgs a = fwd_args(h, slot(k), slot(k + 1), pm, vo, t0 + s0 + k, h->force_scratch,
                                     (long long)h->max_steps * 3, t0 + s0 + k, 0);
                timed(h, K_G2P, s, [&] { launch_g2p(a, h->n_blocks, h->block, s, h->tight, true); });
            }
        } else {
            // recompute the segment, keeping every state and grid; the state
            // after its last substep is not needed by the adjoint
            chain_forward(h, t0 + s0, L, slot, grids, h->force_scratch, (long long)h->max_steps * 3, t0 + s0, 0, true,
                          true, s0, s);
        }
        h->fwd_partial = nullptr;
        h->in_recompute = false;
    };
    auto adjoint = [&](long long sgi, cudaStream_t s) {
        const int s0 = (int)(sgi * K);
        const int L = std::min(K, n - s0);
        auto slot = [&](int j) -> float* { return seg_slot(sgi, j); };
        // adjoint of the state at global step g (relative to t0) lives in A[(n - g) & 1]
        auto adj_args = [&](int k) {
            AdjArgs a;
            a.sc = h->sc;
            a.blk = h->blk;
            a.gblk = h->gblk;
            a.cur = slot(k);
            a.stride = h->stride;
            a.pm = h->pm + grid_slot(sgi, k) * h->G;
            a.vo = h->vo + grid_slot(sgi, k) * h->G;
            a.ga = h->ga;
            a.pmb = h->pmb;
            a.adj_next = A[(n - (s0 + k + 1)) & 1];
            a.adj_cur = A[(n - (s0 + k)) & 1];
            a.traj = h->traj;
            a.traj_len = h->max_steps + 1;
            a.f = t0 + s0 + k;
            a.params = h->params;
            a.models = h->models;
            a.dforce = h->dfbuf;
            a.dforce_stride = (long long)h->max_steps * 3;
            a.fo = s0 + k;
            a.pgrad = h->pgrad;
            a.partial = h->partial;
            a.counters = h->counters;
            a.batch = h->B;
            a.cur2 = nullptr;
            a.vo2 = nullptr;
            a.adj_prev = nullptr;
            a.box = box_slot(h, s0 + k);
            a.lsort = h->lsort;
            a.pdl = h->pdl >= 2;
            a.lstage = h->lstage;
            a.gprio = h->gprio ? h->prio_hi : 0;
            a.pf_dist = h->pf_dist;
            a.n_blocks = h->n_blocks;
            return a;
        };
        if (persist_on(h)) {
            // substeps L-1 .. 0 in launches of up to kSegMax
            for (int k1 = L - 1; k1 >= 0; k1 -= kSegMax) {
                const int nq = std::min(kSegMax, k1 + 1);
                SegAdjArgs g;
                memset(&g, 0, sizeof(g));
                for (int q = 0; q < nq; ++q) {
                    const AdjArgs ak = adj_args(k1 - q);
                    g.cur[q] = ak.cur;
                    g.pm[q] = ak.pm;
                    g.vo[q] = ak.vo;
                    g.adj_next[q] = ak.adj_next;
                    g.adj_cur[q] = ak.adj_cur;
                    g.box[q] = ak.box;
                }
                g.a = adj_args(k1);
                g.a.pdl = 0;
                g.nsteps = nq;
                g.f0 = t0 + s0 + k1;
                g.fo0 = s0 + k1;
                g.n_pblocks = h->n_blocks;
                g.n_gblocks = h->n_gblocks;
                g.bar = h->gbar;
                g.status = h->status;
                g.limit_ns = h->bar_limit_ns;
                g.bar_extra = h->bar_extra;
                cudaMemsetAsync(h->gbar, 0, sizeof(GridBar), s);
                cudaMemsetAsync(h->counters, 0, (size_t)3 * h->B * sizeof(unsigned), s);
                timed(h, K_SEG_ADJ, s, [&] { launch_seg_adj(g, seg_grid(h), h->any_svd, s); });
            }
        } else if (!fused_adj(h)) {
            for (int k = L - 1; k >= 0; --k) run_adj_substep(h, adj_args(k), s, k);
        } else {
            // G2P adjoint of the segment's last substep, then per substep k the
            // grid adjoint and the P2G adjoint of k fused with the G2P adjoint of
            // k-1; the first substep of the segment ends with a plain P2G adjoint
            // that stores the whole state adjoint for the previous segment
            const int var = h->p2g_variant;  // P2G_PLAIN, P2G_VEC or P2G_WARP here
            {
                AdjArgs a = adj_args(L - 1);
                timed(h, K_G2P_ADJ, s, [&] { launch_g2p_adj(a, h->n_blocks, h->block, var, s, h->tight); });
            }
            for (int k = L - 1; k >= 0; --k) {
                AdjArgs a = adj_args(k);
                timed(h, K_GRID_ADJ, s, [&] { launch_grid_adj(a, h->n_gblocks, h->gblock, s); });
                if (k >= 1) {
                    a.cur2 = slot(k - 1);
                    a.vo2 = h->vo + grid_slot(sgi, k - 1) * h->G;
                    a.adj_prev = A[(n - (s0 + k - 1)) & 1];
                    timed(h, K_P2G_ADJ_G2P_ADJ, s,
                          [&] { launch_p2g_adj_g2p_adj(a, h->n_blocks, h->block, var, h->any_svd, s, h->tight); });
                } else {
                    timed(h, K_P2G_ADJ, s, [&] { launch_p2g_adj(a, h->n_blocks, h->block, h->any_svd, s, h->tight); });
                }
            }
        }
        if (h->rec_resort && sgi > 0) {
            // checkpoint sgi was re-sorted from the state that ended segment
            // sgi-1: bring the adjoint of state s0 back to that order (through
            // the other adjoint slot, whose state s0+1 adjoint is spent)
            float* adj0 = A[(n - s0) & 1];
            float* tmp = A[(n - s0 + 1) & 1];
            timed(h, K_OTHER, s, [&] {
                launch_unpermute(adj0, tmp, h->rs_dest + (size_t)sgi * h->stride, h->stride, h->N, s);
            });
            cudaMemcpyAsync(adj0, tmp, sf * sizeof(float), cudaMemcpyDeviceToDevice, s);
        }
    };
    if (!ovl) {
        for (long long sgi = nseg - 1; sgi >= 0; --sgi) {
            recompute(sgi, st);
            adjoint(sgi, st);
        }
    } else {
        // software pipeline over the two streams: the recompute of segment
        // sgi-1 (rstream) overlaps the adjoint of segment sgi (st); it reuses
        // the buffers of segment sgi+1, so it waits for that adjoint first
        cudaStream_t rs = h->rstream;
        cudaEventRecord(h->ev_fork, st);
        cudaStreamWaitEvent(rs, h->ev_fork, 0);
        recompute(nseg - 1, rs);
        cudaEventRecord(h->ev_r[(nseg - 1) & 1], rs);
        for (long long sgi = nseg - 1; sgi >= 0; --sgi) {
            if (sgi >= 1) {
                if (sgi + 1 <= nseg - 1) cudaStreamWaitEvent(rs, h->ev_a[(sgi + 1) & 1], 0);
                recompute(sgi - 1, rs);
                cudaEventRecord(h->ev_r[(sgi - 1) & 1], rs);
            }
            cudaStreamWaitEvent(st, h->ev_r[sgi & 1], 0);
            adjoint(sgi, st);
            cudaEventRecord(h->ev_a[sgi & 1], st);
        }
        cudaEventRecord(h->ev_join, rs);
        cudaStreamWaitEvent(st, h->ev_join, 0);
    }
    cudaMemsetAsync(h->pm, 0, (size_t)h->G * sizeof(float4), st);
    timed(h, K_OTHER, st, [&] { launch_reduce_pgrad(h->pgrad, n, h->B, h->dpbuf, st); });
    return n & 1;
}

}  // namespace

extern "C" {

int dstir_backward(DstirHandle* h, const float* dL_dforce, float* dL_dparams, float* dL_dx0, float* dL_dv0,
                   float* dL_dC0, float* dL_dF0, void* stream) {
    if (!h) return DSTIR_EINVAL;
    if (!h->recorded) return fail(h, DSTIR_ESTATE, "dstir_backward: no recorded forward (record=1) to differentiate");
    if (!dL_dforce) return fail(h, DSTIR_EINVAL, "dstir_backward: dL_dforce is required");
    cudaStream_t st = S(stream);
    const int n = h->rec_n, K = h->rec_K;
    size_t sf = slot_floats(h);
    int rc;
    const bool ovl = overlap_on(h) && (n + K - 1) / K >= 2;
    const long long nbuf = ovl ? 2 : 1;
    if (nbuf * K > h->seg_slots) {
        if ((rc = dalloc(h, &h->seg, (size_t)(nbuf * K) * sf, "segment states"))) return rc;
        h->seg_slots = nbuf * K;
    }
    if (!h->rec_store && (rc = ensure_grid_slots(h, nbuf * K))) return rc;
    if (ovl) {
        if (!h->rstream) {
            CUDA_TRY(h, cudaStreamCreateWithFlags(&h->rstream, cudaStreamNonBlocking));
            cudaEvent_t* evs[] = {&h->ev_fork, &h->ev_join, &h->ev_r[0], &h->ev_r[1], &h->ev_a[0], &h->ev_a[1]};
            for (cudaEvent_t* e : evs) CUDA_TRY(h, cudaEventCreateWithFlags(e, cudaEventDisableTiming));
        }
        if (!h->partial2 && (rc = dalloc(h, &h->partial2, (size_t)h->partial_len * 4, "recompute partial sums")))
            return rc;
    }
    if (binned(h) && (rc = ensure_bin_slots(h, K))) return rc;
    // dL/dforce [B][n][3] -> internal [B][max_steps][3]
    CUDA_TRY(h, cudaMemcpy2DAsync(h->dfbuf, (size_t)h->max_steps * 3 * sizeof(float), dL_dforce,
                                  (size_t)n * 3 * sizeof(float), (size_t)n * 3 * sizeof(float), (size_t)h->B,
                                  cudaMemcpyDeviceToDevice, st));
    long long want[8] = {h->rec_t0, n, K, h->epoch, h->p2g_variant * 16 + h->fuse * 2 + h->fuse_adj,
                         h->block * 4096 + h->gblock,
                         (h->rec_resort ? 1 : 0) + (h->rec_store ? 2 : 0) + (ovl ? 4 : 0) + (h->lsort ? 8 : 0) +
                             16 * h->pdl + 64 * h->lstage + 256 * h->gprio + 512LL * h->pf_dist,
                         0};
    int final_nx = n % 2;
    rc = run_maybe_graph(h, st, &h->bwd_exec, h->bwd_key, want, &h->bwd_kernels,
                         [&](cudaStream_t s2) { enqueue_backward(h, s2); });
    if (rc) return rc;
    float* A[2] = {h->adj, h->adj + sf};
    if (dL_dparams)
        CUDA_TRY(h, cudaMemcpyAsync(dL_dparams, h->dpbuf, (size_t)h->B * 4 * sizeof(float), cudaMemcpyDeviceToDevice,
                                    st));
    if (dL_dx0 || dL_dv0 || dL_dC0 || dL_dF0)
        timed(h, K_OTHER, st,
              [&] {
                  launch_unpack_state(A[final_nx], h->stride, h->N, dL_dx0, dL_dv0, dL_dC0, dL_dF0,
                                      h->rec_perm_id ? nullptr : h->perm_rec0, st);
              });
    CUDA_TRY(h, cudaGetLastError());
    return DSTIR_OK;
}

int dstir_status(DstirHandle* h, uint32_t* flags, void* stream) {
    if (!h || !flags) return DSTIR_EINVAL;
    unsigned v = 0;
    CUDA_TRY(h, cudaMemcpyAsync(&v, h->status, sizeof(unsigned), cudaMemcpyDeviceToHost, S(stream)));
    CUDA_TRY(h, cudaStreamSynchronize(S(stream)));
    CUDA_TRY(h, cudaMemsetAsync(h->status, 0, sizeof(unsigned), S(stream)));
    *flags = v;
    return DSTIR_OK;
}

int dstir_set_option(DstirHandle* h, const char* key, int64_t value) {
    if (!h || !key) return DSTIR_EINVAL;
    if (!strcmp(key, "p2g")) {
        // variant 2 (one thread per binned cell) was measured slower on every
        // shape and retired; its number stays unused
        if (value < 0 || value > 4 || value == 2)
            return fail(h, DSTIR_EINVAL, "p2g variant %lld not in {0, 1, 3, 4}", (long long)value);
        h->p2g_variant = (int)value;
        h->recorded = false;
        return DSTIR_OK;
    }
    if (!strcmp(key, "block") || !strcmp(key, "gblock")) {
        // grid blocks may be larger (fewer partial sums in the rod-force
        // reduction)
        const bool grid_key = !strcmp(key, "gblock");
        if (value != 64 && value != 128 && value != 256 && !(grid_key && (value == 512 || value == 1024)))
            return fail(h, DSTIR_EINVAL, "%s must be 64, 128 or 256 (gblock also 512 or 1024)", key);
        if (!strcmp(key, "block"))
            h->block = (int)value;
        else
            h->gblock = (int)value;
        h->recorded = false;
        return build_tables(h);
    }
    if (!strcmp(key, "graph")) {
        h->use_graph = value ? 1 : 0;
        return DSTIR_OK;
    }
    if (!strcmp(key, "resort")) {
        h->resort = value ? 1 : 0;
        h->recorded = false;
        return DSTIR_OK;
    }
    if (!strcmp(key, "overlap")) {
        h->overlap = value ? 1 : 0;
        return DSTIR_OK;
    }
    if (!strcmp(key, "persist")) {
        if (value && h->seg_grid_max < 0) h->seg_grid_max = seg_max_blocks(h->any_svd);
        if (value && h->seg_grid_max <= 0)
            return fail(h, DSTIR_EINVAL, "persist: cooperative launches are not available on this device");
        int rc;
        if (value && !h->gbar && (rc = dalloc(h, &h->gbar, 1, "grid barrier"))) return rc;
        h->persist = value ? 1 : 0;
        ++h->epoch;
        return DSTIR_OK;
    }
    if (!strcmp(key, "barrier_limit_us")) {
        if (value < 1 || value > 60000000) return fail(h, DSTIR_EINVAL, "barrier_limit_us must be 1..60000000");
        h->bar_limit_ns = value * 1000;
        ++h->epoch;
        return DSTIR_OK;
    }
    if (!strcmp(key, "barrier_test")) {
        h->bar_extra = value ? 1 : 0;
        ++h->epoch;
        return DSTIR_OK;
    }
    if (!strcmp(key, "lsort")) {
        h->lsort = value ? 1 : 0;
        return DSTIR_OK;
    }
    if (!strcmp(key, "lstage")) {
        if (value < 0 || value > 3) return fail(h, DSTIR_EINVAL, "lstage must be 0..3");
        h->lstage = (int)value;
        return DSTIR_OK;
    }
    if (!strcmp(key, "prefetch")) {
        if (value < 0 || value > 100000) return fail(h, DSTIR_EINVAL, "prefetch must be 0..100000");
        h->pf_dist = (int)value;
        return DSTIR_OK;
    }
    if (!strcmp(key, "gprio")) {
        h->gprio = value ? 1 : 0;
        return DSTIR_OK;
    }
    if (!strcmp(key, "pdl")) {
        if (value < 0 || value > 2) return fail(h, DSTIR_EINVAL, "pdl must be 0, 1 or 2");
        h->pdl = (int)value;
        return DSTIR_OK;
    }
    if (!strcmp(key, "store_grids")) {
        h->store_grids = value ? 1 : 0;
        h->recorded = false;
        return DSTIR_OK;
    }
    if (!strcmp(key, "box")) {
        h->use_box = value ? 1 : 0;
        ++h->epoch;
        h->recorded = false;
        return DSTIR_OK;
    }
    if (!strcmp(key, "tight")) {
        if (value < 0 || value > 3) return fail(h, DSTIR_EINVAL, "tight %lld not in 0..3", (long long)value);
        h->tight = (int)value;
        ++h->epoch;
        return DSTIR_OK;
    }
    if (!strcmp(key, "fuse_adj")) {
        h->fuse_adj = value ? 1 : 0;
        h->recorded = false;
        ++h->epoch;
        return DSTIR_OK;
    }
    if (!strcmp(key, "fuse")) {
        h->fuse = value ? 1 : 0;
        h->recorded = false;
        ++h->epoch;
        return DSTIR_OK;
    }
    if (!strcmp(key, "brick_scatter")) {
        if (value < 0 || value > 2) return fail(h, DSTIR_EINVAL, "brick_scatter %lld not in 0..2", (long long)value);
        h->brick_scatter = (int)value;
        h->recorded = false;
        ++h->epoch;
        return DSTIR_OK;
    }
    if (!strcmp(key, "brick_gather")) {
        h->brick_gather = value ? 1 : 0;
        h->recorded = false;
        ++h->epoch;
        return DSTIR_OK;
    }
    if (!strcmp(key, "profile")) {  // 1: time every launch with CUDA events; resets the totals
        h->prof.reset();
        h->prof.on = value != 0;
        return DSTIR_OK;
    }
    if (!strcmp(key, "launches")) {  // reset the launch counter
        h->launches = value;
        return DSTIR_OK;
    }
    return fail(h, DSTIR_EINVAL, "unknown option '%s'", key);
}

int dstir_get_option(const DstirHandle* h, const char* key, int64_t* value) {
    if (!h || !key || !value) return DSTIR_EINVAL;
    if (!strcmp(key, "p2g")) *value = h->p2g_variant;
    else if (!strcmp(key, "block")) *value = h->block;
    else if (!strcmp(key, "gblock")) *value = h->gblock;
    else if (!strcmp(key, "graph")) *value = h->use_graph;
    else if (!strcmp(key, "brick_gather")) *value = h->brick_gather;
    else if (!strcmp(key, "brick_scatter")) *value = h->brick_scatter;
    else if (!strcmp(key, "fuse")) *value = h->fuse;
    else if (!strcmp(key, "fuse_adj")) *value = h->fuse_adj;
    else if (!strcmp(key, "resort")) *value = h->resort;
    else if (!strcmp(key, "tight")) *value = h->tight;
    else if (!strcmp(key, "box")) *value = h->use_box;
    else if (!strcmp(key, "store_grids")) *value = h->store_grids;
    else if (!strcmp(key, "overlap")) *value = h->overlap;
    else if (!strcmp(key, "persist")) *value = h->persist;
    else if (!strcmp(key, "persist_active")) *value = persist_on(h) ? 1 : 0;
    else if (!strcmp(key, "barrier_limit_us")) *value = h->bar_limit_ns / 1000;
    else if (!strcmp(key, "barrier_test")) *value = h->bar_extra;
    else if (!strcmp(key, "lsort")) *value = h->lsort;
    else if (!strcmp(key, "pdl")) *value = h->pdl;
    else if (!strcmp(key, "lstage")) *value = h->lstage;
    else if (!strcmp(key, "gprio")) *value = h->gprio;
    else if (!strcmp(key, "prefetch")) *value = h->pf_dist;
    else if (!strcmp(key, "n_blocks")) *value = h->n_blocks;
    else if (!strcmp(key, "n_gblocks")) *value = h->n_gblocks;
    else if (!strcmp(key, "stride")) *value = h->stride;
    else if (!strcmp(key, "launches")) *value = h->launches;
    else if (!strncmp(key, "prof_ns:", 8) || !strncmp(key, "prof_count:", 11)) {
        // totals of the in-library profiler for one kernel kind ("prof_ns:p2g", "prof_count:p2g")
        bool ns = key[5] == 'n';
        const char* name = key + (ns ? 8 : 11);
        DstirHandle* hm = const_cast<DstirHandle*>(h);
        hm->prof.drain();
        for (int k = 0; k < K_NUM; ++k)
            if (!strcmp(name, kKernelNames[k])) {
                *value = ns ? (int64_t)(hm->prof.total_ms[k] * 1e6) : (int64_t)hm->prof.count[k];
                return DSTIR_OK;
            }
        return DSTIR_EINVAL;
    } else return DSTIR_EINVAL;
    return DSTIR_OK;
}

int dstir_svd3(const float* A, float* U, float* Sg, float* V, int64_t n, void* stream) {
    if (n < 0 || (n > 0 && (!A || !U || !Sg || !V))) return DSTIR_EINVAL;
    launch_svd3(A, U, Sg, V, n, S(stream));
    return cudaGetLastError() == cudaSuccess ? DSTIR_OK : DSTIR_ECUDA;
}

int dstir_svd3_backward(const float* gU, const float* gS, const float* gV, const float* U, const float* Sg,
                        const float* V, float* gA, int64_t n, void* stream) {
    if (n < 0 || (n > 0 && (!gU || !gS || !gV || !U || !Sg || !V || !gA))) return DSTIR_EINVAL;
    launch_svd3_backward(gU, gS, gV, U, Sg, V, gA, n, S(stream));
    return cudaGetLastError() == cudaSuccess ? DSTIR_OK : DSTIR_ECUDA;
}

}  // extern "C"
