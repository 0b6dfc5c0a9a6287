// Allocation-free substep: dstir_substep_static (include/diffstir.h).
//
// Some callers cannot let this library call cudaMalloc.  A host framework that
// owns the device memory pool may forbid allocations from its callbacks, and
// a time-critical stepping loop cannot afford the device-wide synchronisation
// that cudaMalloc / cudaFree may imply.  For them this file runs one MLS-MPM
// substep of one scene (the same P2G, grid-update and G2P kernels as
// dstir_substep) with all of its scratch memory -- the P2G grid, the velocity
// grid, the block tables, the scene constants and the reduction partials -- in
// one file-scope static device array, kScratchBytes (about 8.3 MB) in size.
// Every GPU that loads the library holds that array until the process exits.
//
// Limits: n_grid <= kMaxAxis (64, so at most kMaxNodes grid nodes) and at most
// kMaxParticles particles; larger scenes are rejected with DSTIR_ERANGE before
// anything is queued.
//
// The array is shared by every call: each call clears what must start at zero
// (the P2G grid and the reduction counters) before use, and two calls whose
// work overlaps on the GPU (different streams, or different host threads)
// race on it.  Serialise them.
//
// The array's name is a host-side stand-in, not a device address.  Every call,
// with the caller's device current, asks the runtime for the array's device
// address (cudaGetSymbolAddress: no allocation), so the address stays right
// across a device reset.  The first call on a device may load the module;
// make it before any stream capture.
#include <cuda_runtime.h>

#include <cstring>

#include "common.cuh"
#include "internal.h"

namespace dstir {
namespace {

constexpr int kMaxAxis = 64;
constexpr long long kMaxNodes = (long long)kMaxAxis * kMaxAxis * kMaxAxis;
constexpr long long kMaxParticles = 1LL << 20;
constexpr int kBlock = 256;
constexpr long long kMaxPBlocks = kMaxParticles / kBlock + 3;   // + one partial block per particle kind
constexpr long long kMaxGBlocks = kMaxNodes / kBlock;

constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kOffPm = 0;
constexpr size_t kOffVo = align256(kOffPm + kMaxNodes * sizeof(float4));
constexpr size_t kOffBlk = align256(kOffVo + kMaxNodes * sizeof(float4));
constexpr size_t kOffGblk = align256(kOffBlk + kMaxPBlocks * sizeof(BlockInfo));
constexpr size_t kOffScene = align256(kOffGblk + kMaxGBlocks * sizeof(GridBlock));
constexpr size_t kOffPartial = align256(kOffScene + sizeof(SceneDev));
constexpr size_t kOffMisc = align256(kOffPartial + (kMaxPBlocks > kMaxGBlocks ? kMaxPBlocks : kMaxGBlocks) * 4 * sizeof(float));
// misc: counters[3], status, model, params[4]
constexpr size_t kScratchBytes = align256(kOffMisc + 16 * sizeof(unsigned));

static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

// Device address of the scratch array on the current device.
int scratch_for_current_device(unsigned char** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || p == nullptr) return DSTIR_ECUDA;
    *out = static_cast<unsigned char*>(p);
    return DSTIR_OK;
}

// Fills the block tables, the scene constants and the model index inside the
// scratch (everything by value, so no host buffer has to outlive the call).
__global__ void fill_static_tables(BlockInfo* blk, GridBlock* gblk, SceneDev* sc, int* model, SceneDev sd,
                                   int model_index, long long nl, long long nr, long long nc, int nb0, int nb1,
                                   int nb2, long long G, int ngb) {
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int nb = nb0 + nb1 + nb2;
    if (t == 0) {
        *sc = sd;
        *model = model_index;
    }
    if (t < nb) {
        int b = (int)t, kd, nbk;
        long long start0, cnt;
        if (b < nb0) {
            kd = 0; nbk = nb0; start0 = 0; cnt = nl;
        } else if (b < nb0 + nb1) {
            kd = 1; nbk = nb1; start0 = nl; cnt = nr; b -= nb0;
        } else {
            kd = 2; nbk = nb2; start0 = nl + nr; cnt = nc; b -= nb0 + nb1;
        }
        BlockInfo bi;
        bi.scene = 0;
        bi.kind = kd;
        bi.idx = b;
        bi.count = nbk;
        bi.start = start0 + (long long)b * kBlock;
        bi.end = (start0 + cnt < bi.start + kBlock) ? start0 + cnt : bi.start + kBlock;
        blk[t] = bi;
    }
    if (t < ngb) {
        GridBlock gb;
        gb.scene = 0;
        gb.idx = (int)t;
        gb.count = ngb;
        gb.pad = 0;
        gb.start = t * kBlock;
        gb.end = (G < gb.start + kBlock) ? G : gb.start + kBlock;
        gblk[t] = gb;
    }
}

}  // namespace
}  // namespace dstir

using namespace dstir;

extern "C" int dstir_substep_static(const DstirSceneDesc* scene, const float* params, const float* traj2,
                                    const float* state_in, float* state_out, float* force_out, void* stream) {
    if (!scene || !params || !traj2 || !state_in || !state_out || !force_out) return DSTIR_EINVAL;
    const DstirSceneDesc& d = *scene;
    if (d.n_grid < 4 || d.n_liquid < 0 || d.n_rod < 0 || d.n_container < 0 || d.bound < 0 || !(d.dt > 0.f) ||
        d.model < 0 || d.model > 2 || d.rod_mode < 0 || d.rod_mode > 1 || d.j_mode < 0 || d.j_mode > 1 ||
        (d.rod_mode == DSTIR_ROD_CYLINDER && d.n_rod != 0))
        return DSTIR_EINVAL;
    // per-axis bound first: n_grid^3 is only formed once it cannot overflow
    if (d.n_grid > kMaxAxis) return DSTIR_ERANGE;
    const long long G = (long long)d.n_grid * d.n_grid * d.n_grid;
    const long long N = (long long)d.n_liquid + d.n_rod + d.n_container;
    if (G > kMaxNodes || N > kMaxParticles) return DSTIR_ERANGE;
    if (N == 0) return DSTIR_OK;
    // an error left pending by earlier work on this thread is not ours to
    // clear; report it before queueing anything, so that the checks after our
    // own launches see only our own errors
    if (cudaPeekAtLastError() != cudaSuccess) return DSTIR_ECUDA;
    unsigned char* base = nullptr;
    int rc = scratch_for_current_device(&base);
    if (rc) return rc;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

    // scene constants; fill_static_tables writes them and the block tables into the scratch
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
    sd.p0 = 0;
    sd.goff = 0;
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
    const int nb0 = (int)((d.n_liquid + kBlock - 1) / kBlock), nb1 = (int)((d.n_rod + kBlock - 1) / kBlock),
              nb2 = (int)((d.n_container + kBlock - 1) / kBlock);
    const int nb = nb0 + nb1 + nb2;
    const int ngb = (int)((G + kBlock - 1) / kBlock);
    float4* pm = reinterpret_cast<float4*>(base + kOffPm);
    float4* vo = reinterpret_cast<float4*>(base + kOffVo);
    BlockInfo* blk_d = reinterpret_cast<BlockInfo*>(base + kOffBlk);
    GridBlock* gblk_d = reinterpret_cast<GridBlock*>(base + kOffGblk);
    SceneDev* sc_d = reinterpret_cast<SceneDev*>(base + kOffScene);
    float* partial = reinterpret_cast<float*>(base + kOffPartial);
    unsigned* misc = reinterpret_cast<unsigned*>(base + kOffMisc);
    unsigned* counters = misc;            // [3]
    unsigned* status = misc + 3;          // [1]
    int* model = reinterpret_cast<int*>(misc + 4);
    float* prm = reinterpret_cast<float*>(misc + 8);  // [4]
    const int nt = nb > ngb ? nb : ngb;
    fill_static_tables<<<(nt + 255) / 256, 256, 0, st>>>(blk_d, gblk_d, sc_d, model, sd, d.model, d.n_liquid,
                                                         d.n_rod, d.n_container, nb0, nb1, nb2, G, ngb);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(prm, params, 4 * sizeof(float), cudaMemcpyDeviceToDevice, st);
    // what must start at zero: the P2G grid, the reduction counters and status, the force
    if (e == cudaSuccess) e = cudaMemsetAsync(pm, 0, (size_t)G * sizeof(float4), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(force_out, 0, 3 * sizeof(float), st);
    if (e != cudaSuccess) return DSTIR_ECUDA;

    FwdArgs a;
    a.sc = sc_d;
    a.blk = blk_d;
    a.gblk = gblk_d;
    a.cur = state_in;
    a.next = state_out;
    a.stride = N;
    a.pm = pm;
    a.vo = vo;
    a.traj = traj2;
    a.traj_len = 2;
    a.f = 0;
    a.params = prm;
    a.models = model;
    a.force = force_out;
    a.force_stride = 3;
    a.fo = 0;
    a.partial = partial;
    a.counters = counters;
    a.status = status;
    a.clear_pm = 0;
    a.batch = 1;
    const bool svdj = d.j_mode == DSTIR_J_SVD;
    launch_p2g(a, nb, kBlock, P2G_VEC, svdj, st);
    launch_grid(a, ngb, kBlock, st);
    launch_g2p(a, nb, kBlock, st);
    return cudaGetLastError() == cudaSuccess ? DSTIR_OK : DSTIR_ECUDA;
}
