// Forward and adjoint kernels of one MLS-MPM substep (sm_103a).
//
// Forward substep f (reference forward(s), simulation_functions.py:341-348):
//   p2g_kernel   compute_F_tmp :39-42 + p2g :104-196 (stress, F[f+1], APIC scatter)
//   grid_kernel  grid_op :199-225 (+ moving cylinder rod and its reaction force)
//   g2p_kernel   g2p :228-290 (+ rod reaction force of compute_loss :330-336)
// clear_grid (:3-10) is fused into grid_kernel (it zeroes the P2G grid after
// reading it).  The reference's svd kernel (:55-58) feeds nothing downstream;
// it runs here only when J is taken from the SVD (DSTIR_J_SVD).
//
// Adjoint substep f (the .grad kernels Taichi generated, called in reverse by
// backward(s), :351-365): g2p_adj_kernel (G2P^T: scatter into the grid
// adjoint), grid_adj_kernel (grid_op^T), p2g_adj_kernel (P2G^T: gather, stress
// and F_tmp adjoints, parameter gradient block reduction).
#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"
#include "svd.cuh"
#include "device_util.cuh"
#include "adjoint.cuh"

namespace dstir {

// ---------------------------------------------------------------------------
// forward
// ---------------------------------------------------------------------------
// The kernel bodies below take their block index `vb` as an argument: a
// one-substep kernel passes blockIdx.x, a persistent segment kernel loops its
// blocks over the virtual blocks of each phase (every body ends with no
// pending barrier, and the caller separates two bodies by __syncthreads).
// NC: load policy (ldp in device_util.cuh).  NC is true exactly in the
// one-substep kernels: their bodies read the block descriptor, the scene and
// the other tables written before the rollout, then wait on the previous
// kernel (pdl_enter) before touching the state or the grids.
template <int VARIANT, bool SVDJ, bool NC>
__device__ __forceinline__ void p2g_body(const FwdArgs& a, int vb) {
    __shared__ SceneDev s;
    __shared__ BlockInfo bi;
    __shared__ int boxsh[8][6];
    if (threadIdx.x == 0) {
        bi = a.blk[vb];
        s = a.sc[bi.scene];
    }
    if (NC) pdl_enter();
    __syncthreads();
    constexpr bool WARP = VARIANT == P2G_WARP;
    long long p = bi.start + threadIdx.x;
    bool active = p < bi.end;
    if (!active) p = bi.end - 1;  // the lane computes a copy and writes nothing
    // re-interleaved blocks may stage their state through shared memory
    // (lstage): thread t loads slot t (coalesced, in flight during the sort),
    // thread s then reads the slot it processes; F[f+1] goes back the same way
    __shared__ float pst[WARP ? NS : 1][WARP ? 256 : 1];
    bool staged = false;
    int slot = threadIdx.x;
    if constexpr (WARP) {
        __shared__ LocalOrderSmem lo;
        if (a.lsort && bi.kind == KIND_LIQUID) {
            const int count = (int)(bi.end - bi.start);
            staged = (a.lstage & 1) && blockDim.x <= 256;
            if (staged && (int)threadIdx.x < count)
#pragma unroll
                for (int c = 0; c < NS; ++c) pst[c][threadIdx.x] = ldp<NC>(a.cur + (long long)c * a.stride + p);
            // local_interleave's barriers make the staged state visible
            slot = local_interleave_any(a.cur, a.stride, bi.start, count, s.inv_dx, s.n, lo);
            p = bi.start + slot;
            active = p < bi.end;
            if (!active) {
                p = bi.end - 1;
                slot = count - 1;
            }
        }
    }
    float x[3], v[3], C[9];
    if (staged) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            x[c] = pst[OX + c][slot];
            v[c] = pst[OV + c][slot];
        }
#pragma unroll
        for (int i = 0; i < 9; ++i) C[i] = pst[OC + i][slot];
    } else {
        load3<NC>(a.cur, a.stride, OX, p, x);
        load3<NC>(a.cur, a.stride, OV, p, v);
        load9<NC>(a.cur, a.stride, OC, p, C);
    }
    float m, vv[3], A[9];
    if (bi.kind == KIND_LIQUID) {
        float F[9], prm[4];
        if (staged) {
#pragma unroll
            for (int i = 0; i < 9; ++i) F[i] = pst[OF + i][slot];
        } else {
            load9<NC>(a.cur, a.stride, OF, p, F);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) prm[i] = __ldg(a.params + bi.scene * 4 + i);
        LiquidP2G q;
        liquid_p2g<SVDJ>(s, __ldg(a.models + bi.scene), prm, v, C, F, q);
        if (staged) {  // block-uniform
            __syncthreads();  // every thread has read its staged F
            if (active)
#pragma unroll
                for (int i = 0; i < 9; ++i) pst[OF + i][slot] = q.Ft[i];
            __syncthreads();
            const long long t = bi.start + threadIdx.x;
            if (t < bi.end)
#pragma unroll
                for (int i = 0; i < 9; ++i) a.next[(long long)(OF + i) * a.stride + t] = pst[OF + i][threadIdx.x];
        } else if (active) {
            store9(a.next, a.stride, OF, p, q.Ft);  // F[f+1] = F_tmp (:153)
        }
        m = s.m_liq;
#pragma unroll
        for (int i = 0; i < 9; ++i) A[i] = q.A[i];
#pragma unroll
        for (int c = 0; c < 3; ++c) vv[c] = q.vv[c];
    } else {
        float F[9];
        load9<NC>(a.cur, a.stride, OF, p, F);
        if (active) store9(a.next, a.stride, OF, p, F);
        m = (bi.kind == KIND_ROD) ? s.m_rod : s.m_cont;
#pragma unroll
        for (int i = 0; i < 9; ++i) A[i] = m * C[i];
#pragma unroll
        for (int c = 0; c < 3; ++c) vv[c] = v[c];
    }
    int base[3];
    float fx[3];
    if (!locate(x, s.inv_dx, s.n, base, fx)) {
        if (active) atomicOr(a.status, DSTIR_STATUS_OUT_OF_GRID);
        active = false;
        base[0] = base[1] = base[2] = 0;
        fx[0] = fx[1] = fx[2] = 1.f;
    }
    if (a.box) box_update(a.box + bi.scene * 6, base, active, boxsh);
    float w[3][3];
    bspline(fx, w);
    // factored affine momentum: with dp = (o - fx) dx,
    // m v' + A dp = cc + dx (i A_0 + j A_1 + k A_2),  cc = m v' - dx A fx
    float cc[3], Ad[9];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        cc[q] = m * vv[q] - s.dx * (A[q * 3 + 0] * fx[0] + A[q * 3 + 1] * fx[1] + A[q * 3 + 2] * fx[2]);
#pragma unroll
        for (int b = 0; b < 3; ++b) Ad[q * 3 + b] = s.dx * A[q * 3 + b];
    }
    RunAgg ra;
    if (WARP) ra = run_agg_flags(active ? (base[0] * s.n + base[1]) * s.n + base[2] : run_agg_inactive_key());
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float wij = w[i][0] * w[j][1];
            const int row = node_index(s, base[0] + i, base[1] + j, base[2]);
            float r[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) r[q] = cc[q] + (float)i * Ad[q * 3 + 0] + (float)j * Ad[q * 3 + 1];
            float4 c[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float W = wij * w[k][2];
                float g0 = W * (r[0] + (float)k * Ad[2]);
                float g1 = W * (r[1] + (float)k * Ad[5]);
                float g2 = W * (r[2] + (float)k * Ad[8]);
                float gm = W * m;
                float4* dst = a.pm + row + k;
                if (VARIANT == P2G_PLAIN) {
                    if (active) {
                        float* d = reinterpret_cast<float*>(dst);
                        atomicAdd(d + 0, g0);
                        atomicAdd(d + 1, g1);
                        atomicAdd(d + 2, g2);
                        atomicAdd(d + 3, gm);
                    }
                } else if (VARIANT == P2G_VEC) {
                    if (active) red_add4(dst, g0, g1, g2, gm);
                } else {
                    c[k] = make_float4(g0, g1, g2, gm);
                }
            }
            if (WARP) run_agg_scatter<4>(ra, a.pm + row, c[0], c[1], c[2], active);
        }
}

template <int VARIANT, bool SVDJ, int MINB>
__global__ void __launch_bounds__(256, MINB) p2g_kernel(FwdArgs a) {
    p2g_body<VARIANT, SVDJ, true>(a, blockIdx.x);
}

// Reaction force of the moving cylinder (the rod branch of grid_op
// :212-220 summed as compute_loss :330-336 does for the rod particles), run
// by the extra blocks of grid_kernel, one per scene: the block walks the nodes
// of the rod's bounding column in a fixed order, reduces m (v_rod - v) / dt
// over the nodes inside the cylinder and clears their P2G entries (the node
// blocks leave those to it).  The node blocks carry no reduction, so the ones
// outside the occupied box finish at once.
// Node (i, j, k) inside the moving cylinder (grid_op :212-214).  Both the
// node blocks and the rod-force block classify nodes with this function, in
// round-to-nearest steps that the compiler may not contract, so the two agree
// bit for bit on which of them owns a node's P2G entry.
__device__ __forceinline__ bool in_rod_cylinder(const SceneDev& s, const float rc[3], int i, int j, int k) {
    const float ex = __fsub_rn(__fmul_rn((float)i, s.dx), rc[0]);
    const float ez = __fsub_rn(__fmul_rn((float)k, s.dx), rc[2]);
    return __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ez, ez)) < s.rod_r2 && __fmul_rn((float)j, s.dx) >= rc[1];
}

template <bool LOOP>
__device__ __forceinline__ void rod_force_block(const FwdArgs& a, int scene, SceneDev& s, float (*sh)[4]) {
    load_scene_shared(s, a.sc + scene);
    __syncthreads();
    if (s.rod_mode != DSTIR_ROD_CYLINDER) return;  // block-uniform
    const float* t0 = a.traj + ((long long)scene * a.traj_len + a.f) * 3;
    float rc[3], rodv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        rc[c] = t0[c];
        rodv[c] = (t0[3 + c] - t0[c]) / s.dt;
    }
    if (!LOOP) pdl_enter();  // the P2G entries below are the previous kernel's output
    const int n = s.n;
    const float r = sqrtf(s.rod_r2);
    // bounding column with one node of slack each way; the cylinder test is
    // the node blocks' own and decides
    const int i0 = max(0, (int)floorf((rc[0] - r) * s.inv_dx) - 1), i1 = min(n - 1, (int)ceilf((rc[0] + r) * s.inv_dx) + 1);
    const int k0 = max(0, (int)floorf((rc[2] - r) * s.inv_dx) - 1), k1 = min(n - 1, (int)ceilf((rc[2] + r) * s.inv_dx) + 1);
    const int j0 = max(0, (int)floorf(rc[1] * s.inv_dx) - 1);
    const int ni = i1 - i0 + 1, nk = k1 - k0 + 1, nj = n - j0;
    const int total = (ni > 0 && nk > 0 && nj > 0) ? ni * nk * nj : 0;
    float fsum[3] = {0.f, 0.f, 0.f};
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
        const int ii = i0 + q / (nj * nk), rem = q % (nj * nk), jj = j0 + rem / nk, kk = k0 + rem % nk;
        if (in_rod_cylinder(s, rc, ii, jj, kk)) {
            float4* gp = a.pm + s.goff + ((long long)ii * n + jj) * n + kk;
            const float4 g = *gp;
            if (a.clear_pm) *gp = make_float4(0.f, 0.f, 0.f, 0.f);
            const float inv_m = 1.f / (g.w + 1e-10f);
            fsum[0] += g.w * (rodv[0] - inv_m * g.x) / s.dt;
            fsum[1] += g.w * (rodv[1] - inv_m * g.y) / s.dt;
            fsum[2] += g.w * (rodv[2] - inv_m * g.z) / s.dt;
        }
    }
    block_reduce<3>(fsum, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int c = 0; c < 3; ++c) a.force[scene * a.force_stride + (long long)a.fo * 3 + c] = fsum[c];
}

// Grid update of the nodes of virtual block vb, or the rod force of one scene
// for vb >= n_gblocks.  LOOP: the block's threads loop over the node block's
// nodes (a persistent kernel, whose blocks may be smaller than the node
// blocks); otherwise one thread per node.
// A one-substep launch may start while the P2G it follows is still running
// (programmatic dependent launch).  The block table, the scene and the
// trajectory are written before the rollout and never by that kernel, so
// they are read before pdl_enter; the occupied box and the node's P2G entry
// are read right after it, both in flight before the block's barrier.
template <bool LOOP>
__device__ __forceinline__ void grid_body(const FwdArgs& a, int vb) {
    __shared__ SceneDev s;
    __shared__ float rc[3], rc1[3];
    __shared__ float sh[32][4];
    __shared__ int bx[6];
    if (vb >= a.n_gblocks) {  // block-uniform: a rod-force block
        rod_force_block<LOOP>(a, vb - a.n_gblocks, s, sh);
        return;
    }
    // every thread reads the block descriptor (one broadcast load), so the
    // scene copy and the trajectory loads do not wait on a serial chain
    const GridBlock gb = a.gblk[vb];
    load_scene_shared(s, a.sc + gb.scene);
    if (threadIdx.x < 3) {
        const float* t0 = a.traj + ((long long)gb.scene * a.traj_len + a.f) * 3;
        rc[threadIdx.x] = t0[threadIdx.x];
        rc1[threadIdx.x] = t0[3 + threadIdx.x];
    }
    if (!LOOP) pdl_enter();
    const bool use_box = a.box != nullptr;
    if (use_box && threadIdx.x < 6) bx[threadIdx.x] = a.box[gb.scene * 6 + threadIdx.x];
    const long long node0 = gb.start + threadIdx.x;
    float4 g0 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!LOOP && node0 < gb.end) g0 = a.pm[node0];
    __syncthreads();
    const int n = s.n;
    auto node_fn = [&](long long node, float4 g) {
        int i, j, k;
        node_ijk((int)(node - s.goff), n, i, j, k);
        // nodes outside the occupied box hold no mass and no stencil reads them:
        // their P2G entry is still zero and their velocity is never gathered
        if (!use_box || box_inside(bx, i, j, k)) {
            // nodes inside the rod belong to the rod-force block, which reads
            // and clears their P2G entries (their velocity is the rod's anyway)
            const bool in_rod = s.rod_mode == DSTIR_ROD_CYLINDER && in_rod_cylinder(s, rc, i, j, k);
            if (a.clear_pm && !in_rod) a.pm[node] = make_float4(0.f, 0.f, 0.f, 0.f);
            float inv_m = 1.f / (g.w + 1e-10f);
            float v[3] = {inv_m * g.x, inv_m * g.y, inv_m * g.z};
            if (s.container_wall) {  // :204-210
                float d0 = (float)i * s.dx - s.ccx, d2 = (float)k * s.dx - s.ccz;
                float n2 = d0 * d0 + d2 * d2;
                if (n2 > s.cr2) {
                    float inv = 1.f / sqrtf(n2);
                    float u0 = d0 * inv, u2 = d2 * inv;
                    float dot = v[0] * u0 + v[2] * u2;
                    v[0] -= u0 * dot;
                    v[2] -= u2 * dot;
                }
            }
            int b = s.bound;  // :211-224
            if (i < b && v[0] < 0.f) v[0] = 0.f;
            if (i > n - b && v[0] > 0.f) v[0] = 0.f;
            if (k < b && v[2] < 0.f) v[2] = 0.f;
            if (k > n - b && v[2] > 0.f) v[2] = 0.f;
            if (j < b && v[1] < 0.f) v[1] = 0.f;
            if (j > n - b && v[1] > 0.f) v[0] = v[1] = v[2] = 0.f;
            if (in_rod)
#pragma unroll
                for (int c = 0; c < 3; ++c) v[c] = (rc1[c] - rc[c]) / s.dt;
            a.vo[node] = make_float4(v[0], v[1], v[2], 0.f);
        }
    };
    if (LOOP) {
        for (long long node = node0; node < gb.end; node += blockDim.x) node_fn(node, a.pm[node]);
    } else if (node0 < gb.end) {
        node_fn(node0, g0);
    }
}

__global__ void __launch_bounds__(1024) grid_kernel(FwdArgs a) {
    grid_body<false>(a, blockIdx.x);  // waits on the previous kernel itself
}

// WRITE_F: also write F of the next state, F_tmp = (I + dt C) F of the
// current one (what P2G stores, :39-42, :153), for the reverse pass's state
// recompute when the P2G grids of the rollout were kept and P2G is not rerun.
template <bool WRITE_F, bool NC>
__device__ __forceinline__ void g2p_body(const FwdArgs& a, int vb) {
    __shared__ SceneDev s;
    __shared__ BlockInfo bi;
    __shared__ float sh[32][4];
    __shared__ float tv[3];
    if (threadIdx.x == 0) {
        bi = a.blk[vb];
        s = a.sc[bi.scene];
        const float* t0 = a.traj + ((long long)bi.scene * a.traj_len + a.f) * 3;
        for (int c = 0; c < 3; ++c) tv[c] = (t0[3 + c] - t0[c]) / s.dt;
    }
    if (NC) pdl_enter();
    __syncthreads();
    long long p = bi.start + threadIdx.x;
    bool active = p < bi.end;
    float dv[3] = {0.f, 0.f, 0.f};
    if (active) {
            float x[3];
        load3<NC>(a.cur, a.stride, OX, p, x);
        int base[3];
        float fx[3];
        float nv[3] = {0.f, 0.f, 0.f};
        float nC[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) nC[i] = 0.f;
        if (locate(x, s.inv_dx, s.n, base, fx)) {
            float w[3][3];
            bspline(fx, w);
            // nC accumulates sum W g o^T (o = node offset); the -fx part is
            // applied once after the loop: sum W g (o - fx)^T = nC - nv fx^T
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const long long row = node_index64(s, base[0] + i, base[1] + j, base[2]);
                    float wij = w[i][0] * w[j][1];
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        float4 g = ldp<NC>(a.vo + row + k);
                        float W = wij * w[k][2];
                        float wg[3] = {W * g.x, W * g.y, W * g.z};
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            nv[q] += wg[q];
                            if (i) nC[q * 3 + 0] += (float)i * wg[q];
                            if (j) nC[q * 3 + 1] += (float)j * wg[q];
                            if (k) nC[q * 3 + 2] += (float)k * wg[q];
                        }
                    }
                }
            float c4 = 4.f * s.inv_dx;
#pragma unroll
            for (int q = 0; q < 3; ++q)
#pragma unroll
                for (int b = 0; b < 3; ++b) nC[q * 3 + b] = c4 * (nC[q * 3 + b] - nv[q] * fx[b]);
        } else {
            atomicOr(a.status, DSTIR_STATUS_OUT_OF_GRID);
        }
        if (WRITE_F) {
            float Cc[9], F[9], Ft[9];
            load9<NC>(a.cur, a.stride, OC, p, Cc);
            load9<NC>(a.cur, a.stride, OF, p, F);
            if (bi.kind == KIND_LIQUID) {
                float IC[9];
#pragma unroll
                for (int i = 0; i < 9; ++i) IC[i] = s.dt * Cc[i] + ((i % 4 == 0) ? 1.f : 0.f);
                matmul3(IC, F, Ft);
            } else {
#pragma unroll
                for (int i = 0; i < 9; ++i) Ft[i] = F[i];
            }
            store9(a.next, a.stride, OF, p, Ft);
        }
        store9(a.next, a.stride, OC, p, nC);
        float nx[3], outv[3];
        if (bi.kind == KIND_LIQUID) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                outv[c] = nv[c];
                nx[c] = x[c] + s.dt * nv[c];
            }
            bool fin = isfinite(nx[0]) && isfinite(nx[1]) && isfinite(nx[2]) && isfinite(nv[0]) &&
                       isfinite(nv[1]) && isfinite(nv[2]);
#pragma unroll
            for (int i = 0; i < 9; ++i) fin = fin && isfinite(nC[i]);
            if (!fin) atomicOr(a.status, DSTIR_STATUS_NAN);
        } else if (bi.kind == KIND_ROD) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                dv[c] = tv[c] - nv[c];  // :267
                outv[c] = tv[c];
                nx[c] = x[c] + tv[c] * s.dt;
            }
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                outv[c] = 0.f;
                nx[c] = x[c];
            }
        }
        store3(a.next, a.stride, OV, p, outv);
        store3(a.next, a.stride, OX, p, nx);
    }
    if (bi.kind == KIND_ROD && s.rod_mode == DSTIR_ROD_PARTICLES) {
        group_sum<3>(dv, sh, a.partial, a.counters + a.batch + bi.scene, vb - bi.idx, bi.count,
                     a.force + bi.scene * a.force_stride + (long long)a.fo * 3, s.force_scale, vb);
    }
}

template <int MINB, bool WRITE_F>
__global__ void __launch_bounds__(256, MINB) g2p_kernel(FwdArgs a) {
    g2p_body<WRITE_F, true>(a, blockIdx.x);
}

// G2P of substep f fused with P2G of substep f+1 (one thread per particle).
// The G2P half is g2p_kernel; its new x, v, C stay in registers for the
// stress of substep f+1 (compute_F_tmp :39-42 with F[f+1] read back, p2g
// :104-196), which scatters into the next grid.  Saves a pass over the
// particle state and a launch per substep.
template <int VARIANT, bool SVDJ, int MINB>
__global__ void __launch_bounds__(256, MINB) g2p_p2g_kernel(FwdArgs a) {
    pdl_enter();
    __shared__ SceneDev s;
    __shared__ BlockInfo bi;
    __shared__ float sh[32][4];
    __shared__ float tv[3];
    __shared__ float prm[4];
    __shared__ int model;
    __shared__ int boxsh[8][6];
    if (threadIdx.x == 0) {
        bi = a.blk[blockIdx.x];
        s = a.sc[bi.scene];
        const float* t0 = a.traj + ((long long)bi.scene * a.traj_len + a.f) * 3;
        for (int c = 0; c < 3; ++c) tv[c] = (t0[3 + c] - t0[c]) / s.dt;
        for (int i = 0; i < 4; ++i) prm[i] = a.params[bi.scene * 4 + i];
        model = a.models[bi.scene];
    }
    __syncthreads();
    constexpr bool WARP = VARIANT == P2G_WARP;
    long long p = bi.start + threadIdx.x;
    bool active = p < bi.end;
    if (!active) p = bi.end - 1;  // the lane computes a copy and writes nothing
    float dv[3] = {0.f, 0.f, 0.f};
    {
        // ---- G2P of substep f
        float x[3];
        load3(a.cur, a.stride, OX, p, x);
        int base[3];
        float fx[3];
        float nv[3] = {0.f, 0.f, 0.f}, nC[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) nC[i] = 0.f;
        if (locate(x, s.inv_dx, s.n, base, fx)) {
            float w[3][3];
            bspline(fx, w);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const int row = node_index(s, base[0] + i, base[1] + j, base[2]);
                    float wij = w[i][0] * w[j][1];
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        float4 g = __ldg(a.vo + row + k);
                        float W = wij * w[k][2];
                        float wg[3] = {W * g.x, W * g.y, W * g.z};
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            nv[q] += wg[q];
                            if (i) nC[q * 3 + 0] += (float)i * wg[q];
                            if (j) nC[q * 3 + 1] += (float)j * wg[q];
                            if (k) nC[q * 3 + 2] += (float)k * wg[q];
                        }
                    }
                }
            float c4 = 4.f * s.inv_dx;
#pragma unroll
            for (int q = 0; q < 3; ++q)
#pragma unroll
                for (int b = 0; b < 3; ++b) nC[q * 3 + b] = c4 * (nC[q * 3 + b] - nv[q] * fx[b]);
        } else if (active) {
            atomicOr(a.status, DSTIR_STATUS_OUT_OF_GRID);
        }
        float vn[3];
        if (bi.kind == KIND_LIQUID) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                vn[c] = nv[c];
                x[c] = x[c] + s.dt * nv[c];
            }
            bool fin = isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]) && isfinite(nv[0]) && isfinite(nv[1]) &&
                       isfinite(nv[2]);
#pragma unroll
            for (int i = 0; i < 9; ++i) fin = fin && isfinite(nC[i]);
            if (!fin && active) atomicOr(a.status, DSTIR_STATUS_NAN);
        } else if (bi.kind == KIND_ROD) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                dv[c] = active ? tv[c] - nv[c] : 0.f;
                vn[c] = tv[c];
                x[c] = x[c] + tv[c] * s.dt;
            }
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) vn[c] = 0.f;
        }
        // ---- P2G of substep f+1 from (x, vn, nC) and F[f+1]
        float F[9];
        load9(a.next, a.stride, OF, p, F);
        if (active) {
            store9(a.next, a.stride, OC, p, nC);
            store3(a.next, a.stride, OV, p, vn);
            store3(a.next, a.stride, OX, p, x);
        }
        float m, mv[3], A[9];
        if (bi.kind == KIND_LIQUID) {
            LiquidP2G q;
            liquid_p2g<SVDJ>(s, model, prm, vn, nC, F, q);
            if (active) store9(a.next2, a.stride, OF, p, q.Ft);
            m = s.m_liq;
#pragma unroll
            for (int i = 0; i < 9; ++i) A[i] = q.A[i];
#pragma unroll
            for (int c = 0; c < 3; ++c) mv[c] = m * q.vv[c];
        } else {
            if (active) store9(a.next2, a.stride, OF, p, F);
            m = (bi.kind == KIND_ROD) ? s.m_rod : s.m_cont;
#pragma unroll
            for (int i = 0; i < 9; ++i) A[i] = m * nC[i];
#pragma unroll
            for (int c = 0; c < 3; ++c) mv[c] = m * vn[c];
        }
        bool in2 = locate(x, s.inv_dx, s.n, base, fx);
        if (!in2 && active) atomicOr(a.status, DSTIR_STATUS_OUT_OF_GRID);
        bool act2 = active && in2;
        if (!in2) {
            base[0] = base[1] = base[2] = 0;
            fx[0] = fx[1] = fx[2] = 1.f;
        }
        if (a.box_next) box_update(a.box_next + bi.scene * 6, base, act2, boxsh);
        {
            float w[3][3];
            bspline(fx, w);
            // factored affine momentum, as in p2g_kernel
            float cc[3], Ad[9];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                cc[q] = mv[q] - s.dx * (A[q * 3 + 0] * fx[0] + A[q * 3 + 1] * fx[1] + A[q * 3 + 2] * fx[2]);
#pragma unroll
                for (int b = 0; b < 3; ++b) Ad[q * 3 + b] = s.dx * A[q * 3 + b];
            }
            RunAgg ra;
            if (WARP) ra = run_agg_flags(act2 ? (base[0] * s.n + base[1]) * s.n + base[2] : run_agg_inactive_key());
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    float wij = w[i][0] * w[j][1];
                    const int row = node_index(s, base[0] + i, base[1] + j, base[2]);
                    float r[3];
#pragma unroll
                    for (int q = 0; q < 3; ++q) r[q] = cc[q] + (float)i * Ad[q * 3 + 0] + (float)j * Ad[q * 3 + 1];
                    float4 c[3];
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        float W = wij * w[k][2];
                        float g0 = W * (r[0] + (float)k * Ad[2]);
                        float g1 = W * (r[1] + (float)k * Ad[5]);
                        float g2 = W * (r[2] + (float)k * Ad[8]);
                        float gm = W * m;
                        float4* dst = a.pm_next + row + k;
                        if (VARIANT == P2G_PLAIN) {
                            if (act2) {
                                float* d = reinterpret_cast<float*>(dst);
                                atomicAdd(d + 0, g0);
                                atomicAdd(d + 1, g1);
                                atomicAdd(d + 2, g2);
                                atomicAdd(d + 3, gm);
                            }
                        } else if (VARIANT == P2G_VEC) {
                            if (act2) red_add4(dst, g0, g1, g2, gm);
                        } else {
                            c[k] = make_float4(g0, g1, g2, gm);
                        }
                    }
                    if (WARP) run_agg_scatter<4>(ra, a.pm_next + row, c[0], c[1], c[2], act2);
                }
        }
    }
    if (bi.kind == KIND_ROD && s.rod_mode == DSTIR_ROD_PARTICLES) {
        group_sum<3>(dv, sh, a.partial, a.counters + a.batch + bi.scene, blockIdx.x - bi.idx, bi.count,
                     a.force + bi.scene * a.force_stride + (long long)a.fo * 3, s.force_scale, blockIdx.x);
    }
}

// ---------------------------------------------------------------------------
// adjoint
// ---------------------------------------------------------------------------
template <int VARIANT, bool NC>
__device__ __forceinline__ void g2p_adj_body(const AdjArgs& a, int vb) {
    __shared__ SceneDev s;
    __shared__ BlockInfo bi;
    __shared__ float fb[3];
    if (threadIdx.x == 0) {
        bi = a.blk[vb];
        s = a.sc[bi.scene];
        const float* d = a.dforce + bi.scene * a.dforce_stride + (long long)a.fo * 3;
        for (int c = 0; c < 3; ++c) fb[c] = d[c];
    }
    if (NC) pdl_enter();
    if (a.pf_dist && vb + a.pf_dist < a.n_blocks) {
        const BlockInfo nb = a.blk[vb + a.pf_dist];
        prefetch_state_l2(a.cur, a.stride, nb.start, nb.end, OX, 3);
        prefetch_state_l2(a.adj_next, a.stride, nb.start, nb.end, 0, 15);
    }
    __syncthreads();
    constexpr bool WARP = VARIANT == P2G_WARP;
    long long p = bi.start + threadIdx.x;
    bool active = p < bi.end;
    if (!WARP && !active) return;
    if (!active) p = bi.end - 1;  // WARP: the lane computes a copy and scatters nothing
    // re-interleaved blocks may stage their inputs through shared memory
    // (lstage, as in P2G): row c < 3 holds x of the state, row 3 + c
    // component c of the next state's adjoint; rows 0-2 later carry the
    // position adjoint back
    __shared__ float ast[WARP ? 18 : 1][WARP ? 256 : 1];
    bool staged = false;
    int slot = threadIdx.x;
    if constexpr (WARP) {
        __shared__ LocalOrderSmem lo;
        if (a.lsort && bi.kind == KIND_LIQUID) {
            const int count = (int)(bi.end - bi.start);
            staged = (a.lstage & 2) && blockDim.x <= 256;
            if (staged && (int)threadIdx.x < count) {
#pragma unroll
                for (int c = 0; c < 3; ++c) ast[c][threadIdx.x] = ldp<NC>(a.cur + (long long)(OX + c) * a.stride + p);
#pragma unroll
                for (int c = 0; c < 15; ++c) ast[3 + c][threadIdx.x] = a.adj_next[(long long)c * a.stride + p];
            }
            // local_interleave's barriers make the staged inputs visible
            slot = local_interleave_any(a.cur, a.stride, bi.start, count, s.inv_dx, s.n, lo);
            p = bi.start + slot;
            active = p < bi.end;
            if (!active) {
                p = bi.end - 1;
                slot = count - 1;
            }
        }
    }
    float x[3];
    float xb[3] = {0.f, 0.f, 0.f}, vnb[3], Cb[9];
    if (staged) {
#pragma unroll
        for (int c = 0; c < 3; ++c) x[c] = ast[OX + c][slot];
#pragma unroll
        for (int i = 0; i < 9; ++i) Cb[i] = ast[3 + OC + i][slot];
    } else {
        load3<NC>(a.cur, a.stride, OX, p, x);
        load9<NC>(a.adj_next, a.stride, OC, p, Cb);
    }
    if (bi.kind == KIND_LIQUID) {
        float ax[3], av[3];
        if (staged) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                ax[c] = ast[3 + OX + c][slot];
                av[c] = ast[3 + OV + c][slot];
            }
        } else {
            load3<NC>(a.adj_next, a.stride, OX, p, ax);
            load3<NC>(a.adj_next, a.stride, OV, p, av);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            vnb[c] = av[c] + s.dt * ax[c];  // x[f+1] = x[f] + dt*v[f+1] (:247)
            xb[c] = ax[c];
        }
    } else if (bi.kind == KIND_ROD && s.rod_mode == DSTIR_ROD_PARTICLES) {
#pragma unroll
        for (int c = 0; c < 3; ++c) vnb[c] = -fb[c] * s.force_scale;  // dv = v_pres - v_grid
    } else {
        vnb[0] = vnb[1] = vnb[2] = 0.f;
    }
    int base[3];
    float fx[3];
    bool inside = locate(x, s.inv_dx, s.n, base, fx);
    if (WARP && !inside) {
        active = false;
        base[0] = base[1] = base[2] = 0;
        fx[0] = fx[1] = fx[2] = 1.f;
    }
    if (inside || WARP) {
        float w[3][3], dw[3][3];
        bspline_d(fx, w, dw);
        RunAgg ra;
        if (WARP) ra = run_agg_flags(active ? (base[0] * s.n + base[1]) * s.n + base[2] : run_agg_inactive_key());
        // Factored form: with d = o - fx, vnb + c4 Cb d = e + Cc o, where
        // Cc = c4 Cb and e = vnb - Cc fx; the fx-gradient term
        // -c4 W Cb^T g summed over the nodes is -Cc^T U with U = sum W g.
        const float c4 = 4.f * s.inv_dx;
        float Cc[9], e[3];
#pragma unroll
        for (int q = 0; q < 9; ++q) Cc[q] = c4 * Cb[q];
#pragma unroll
        for (int q = 0; q < 3; ++q) e[q] = vnb[q] - (Cc[q * 3 + 0] * fx[0] + Cc[q * 3 + 1] * fx[1] + Cc[q * 3 + 2] * fx[2]);
        float fxb[3] = {0.f, 0.f, 0.f}, U[3] = {0.f, 0.f, 0.f};
        const bool liquid = bi.kind == KIND_LIQUID;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int row = node_index(s, base[0] + i, base[1] + j, base[2]);
                const float wij = w[i][0] * w[j][1], dxij = dw[i][0] * w[j][1], dyij = w[i][0] * dw[j][1];
                float r[3];
#pragma unroll
                for (int q = 0; q < 3; ++q) r[q] = e[q] + (float)i * Cc[q * 3 + 0] + (float)j * Cc[q * 3 + 1];
                float4 cw[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float W = wij * w[k][2];
                    const float rk0 = r[0] + (float)k * Cc[2], rk1 = r[1] + (float)k * Cc[5],
                                rk2 = r[2] + (float)k * Cc[8];
                    float4* dst = a.ga + row + k;
                    const float g0 = W * rk0, g1 = W * rk1, g2 = W * rk2;
                    if (VARIANT == P2G_PLAIN) {
                        float* dd = reinterpret_cast<float*>(dst);
                        atomicAdd(dd + 0, g0);
                        atomicAdd(dd + 1, g1);
                        atomicAdd(dd + 2, g2);
                    } else if (VARIANT == P2G_VEC) {
                        red_add4(dst, g0, g1, g2, 0.f);
                    } else {
                        cw[k] = make_float4(g0, g1, g2, 0.f);
                    }
                    if (liquid) {
                        const float4 g = ldp<NC>(a.vo + row + k);
                        const float Wb = g.x * rk0 + g.y * rk1 + g.z * rk2;
                        U[0] += W * g.x;
                        U[1] += W * g.y;
                        U[2] += W * g.z;
                        fxb[0] += Wb * dxij * w[k][2];
                        fxb[1] += Wb * dyij * w[k][2];
                        fxb[2] += Wb * wij * dw[k][2];
                    }
                }
                if (WARP) run_agg_scatter<3>(ra, a.ga + row, cw[0], cw[1], cw[2], active);
            }
        if (liquid)
#pragma unroll
            for (int b = 0; b < 3; ++b)
                xb[b] += s.inv_dx * (fxb[b] - (Cc[0 * 3 + b] * U[0] + Cc[1 * 3 + b] * U[1] + Cc[2 * 3 + b] * U[2]));
    }
    if (staged) {  // block-uniform
        __syncthreads();  // every thread has read its staged inputs
        if (active)
#pragma unroll
            for (int c = 0; c < 3; ++c) ast[c][slot] = xb[c];
        __syncthreads();
        const long long t = bi.start + threadIdx.x;
        if (t < bi.end)
#pragma unroll
            for (int c = 0; c < 3; ++c) a.adj_cur[(long long)(OX + c) * a.stride + t] = ast[c][threadIdx.x];
    } else if (bi.kind == KIND_LIQUID && active) {
        store3(a.adj_cur, a.stride, OX, p, xb);
    }
}

template <int VARIANT, int MINB>
__global__ void __launch_bounds__(256, MINB) g2p_adj_kernel(AdjArgs a) {
    g2p_adj_body<VARIANT, true>(a, blockIdx.x);
}

// Grid adjoint of the nodes of virtual block vb (LOOP, and the reads before
// pdl_enter: see grid_body; dL/dforce is copied in before the reverse pass).
template <bool LOOP>
__device__ __forceinline__ void grid_adj_body(const AdjArgs& a, int vb) {
    __shared__ SceneDev s;
    __shared__ float rc[3], rc1[3], fb[3];
    __shared__ int bx[6];
    const GridBlock gb = a.gblk[vb];
    load_scene_shared(s, a.sc + gb.scene);
    if (threadIdx.x < 3) {
        const int c = threadIdx.x;
        const float* t0 = a.traj + ((long long)gb.scene * a.traj_len + a.f) * 3;
        const float* d = a.dforce + gb.scene * a.dforce_stride + (long long)a.fo * 3;
        rc[c] = t0[c];
        rc1[c] = t0[3 + c];
        fb[c] = d[c];
    }
    if (!LOOP) pdl_enter();
    const bool use_box = a.box != nullptr;
    if (use_box && threadIdx.x < 6) bx[threadIdx.x] = a.box[gb.scene * 6 + threadIdx.x];
    const long long node0 = gb.start + threadIdx.x;
    float4 g0 = make_float4(0.f, 0.f, 0.f, 0.f), b0 = g0;
    if (!LOOP && node0 < gb.end) {
        g0 = a.pm[node0];
        b0 = a.ga[node0];
    }
    __syncthreads();
    const int n = s.n;
    auto node_fn = [&](long long node, float4 g, float4 vb4) {
        int i, j, k;
        node_ijk((int)(node - s.goff), n, i, j, k);
        // outside the occupied box the velocity adjoint is zero (no stencil
        // scattered there) and no stencil gathers the P/M adjoint
        if (use_box && !box_inside(bx, i, j, k)) return;
        a.ga[node] = make_float4(0.f, 0.f, 0.f, 0.f);
        float inv_m = 1.f / (g.w + 1e-10f);
        float u[3] = {inv_m * g.x, inv_m * g.y, inv_m * g.z};
        float v[3] = {u[0], u[1], u[2]};
        bool proj = false;
        float u0 = 0.f, u2 = 0.f;
        if (s.container_wall) {
            float d0 = (float)i * s.dx - s.ccx, d2 = (float)k * s.dx - s.ccz;
            float n2 = d0 * d0 + d2 * d2;
            if (n2 > s.cr2) {
                float inv = 1.f / sqrtf(n2);
                u0 = d0 * inv;
                u2 = d2 * inv;
                float dot = v[0] * u0 + v[2] * u2;
                v[0] -= u0 * dot;
                v[2] -= u2 * dot;
                proj = true;
            }
        }
        float mask[3] = {1.f, 1.f, 1.f};
        int b = s.bound;
        if (i < b && v[0] < 0.f) { v[0] = 0.f; mask[0] = 0.f; }
        if (i > n - b && v[0] > 0.f) { v[0] = 0.f; mask[0] = 0.f; }
        if (k < b && v[2] < 0.f) { v[2] = 0.f; mask[2] = 0.f; }
        if (k > n - b && v[2] > 0.f) { v[2] = 0.f; mask[2] = 0.f; }
        if (j < b && v[1] < 0.f) { v[1] = 0.f; mask[1] = 0.f; }
        if (j > n - b && v[1] > 0.f) { mask[0] = mask[1] = mask[2] = 0.f; }
        bool inside = false;
        if (s.rod_mode == DSTIR_ROD_CYLINDER) {
            inside = in_rod_cylinder(s, rc, i, j, k);  // the forward's classification
        }
        float ub[3], mb = 0.f;
        if (inside) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float rodv = (rc1[c] - rc[c]) / s.dt;
                ub[c] = -g.w * fb[c] / s.dt;
                mb += fb[c] * (rodv - u[c]) / s.dt;
            }
        } else {
            ub[0] = mask[0] * vb4.x;
            ub[1] = mask[1] * vb4.y;
            ub[2] = mask[2] * vb4.z;
            if (proj) {
                float dot = ub[0] * u0 + ub[2] * u2;
                ub[0] -= u0 * dot;
                ub[2] -= u2 * dot;
            }
        }
        float Pu = g.x * ub[0] + g.y * ub[1] + g.z * ub[2];
        a.pmb[node] = make_float4(inv_m * ub[0], inv_m * ub[1], inv_m * ub[2], mb - inv_m * inv_m * Pu);
    };
    if (LOOP) {
        for (long long node = node0; node < gb.end; node += blockDim.x) node_fn(node, a.pm[node], a.ga[node]);
    } else if (node0 < gb.end) {
        node_fn(node0, g0, b0);
    }
}

__global__ void __launch_bounds__(1024) grid_adj_kernel(AdjArgs a) {
    grid_adj_body<false>(a, blockIdx.x);  // waits on the previous kernel itself
}

// P2G adjoint, one thread per particle (pieces in adjoint.cuh).
template <bool SVDJ, bool NC>
__device__ __forceinline__ void p2g_adj_body(const AdjArgs& a, int vb) {
    __shared__ SceneDev s;
    __shared__ BlockInfo bi;
    __shared__ float sh[32][4];
    __shared__ float prm[4];
    __shared__ int model;
    if (threadIdx.x == 0) {
        bi = a.blk[vb];
        s = a.sc[bi.scene];
        for (int i = 0; i < 4; ++i) prm[i] = a.params[bi.scene * 4 + i];
        model = a.models[bi.scene];
    }
    if (NC) pdl_enter();
    if (a.pf_dist && vb + a.pf_dist < a.n_blocks) {
        const BlockInfo nb = a.blk[vb + a.pf_dist];
        prefetch_state_l2(a.cur, a.stride, nb.start, nb.end, 0, NS);
        prefetch_state_l2(a.adj_next, a.stride, nb.start, nb.end, OF, 9);
    }
    __syncthreads();
    long long p = bi.start + threadIdx.x;
    float pg[4] = {0.f, 0.f, 0.f, 0.f};
    if (p < bi.end) {
        const bool liquid = bi.kind == KIND_LIQUID;
        float x[3];
        load3<NC>(a.cur, a.stride, OX, p, x);
        float m, mv[3], A[9];
        p2g_adj_affine<SVDJ, NC>(a.cur, a.stride, s, prm, model, p, bi.kind, m, mv, A);
        float Ab[9], vvb[3] = {0.f, 0.f, 0.f}, fxb[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int i = 0; i < 9; ++i) Ab[i] = 0.f;
        int base[3];
        float fx[3];
        if (locate(x, s.inv_dx, s.n, base, fx)) {
            float w[3][3], dw[3][3];
            bspline_d(fx, w, dw);
            p2g_adj_gather<NC>(a.pmb, s, base, fx, w, dw, m, mv, A, liquid, Ab, vvb, fxb);
        }
        p2g_adj_finish<SVDJ, NC>(a, s, prm, model, p, bi.kind, m, Ab, vvb, fxb, pg);
    }
    if (bi.kind == KIND_LIQUID) {
        group_sum<4>(pg, sh, a.partial, a.counters + 2 * a.batch + bi.scene, vb - bi.idx, bi.count,
                     a.pgrad + ((long long)a.fo * a.batch + bi.scene) * 4, 1.f, vb);
    }
}

template <bool SVDJ, int MINB>
__global__ void __launch_bounds__(256, MINB) p2g_adj_kernel(AdjArgs a) {
    p2g_adj_body<SVDJ, true>(a, blockIdx.x);
}

// P2G adjoint of substep f fused with the G2P adjoint of substep f-1.  The
// state adjoint of f (x, v, C parts) goes from the first half to the second
// in registers; only its F part (read by the P2G adjoint of f-1) and the
// position-adjoint part of f-1 are stored.
template <int VARIANT, bool SVDJ, int MINB>
__global__ void __launch_bounds__(256, MINB) p2g_adj_g2p_adj_kernel(AdjArgs a) {
    pdl_enter();
    __shared__ SceneDev s;
    __shared__ BlockInfo bi;
    __shared__ float sh[32][4];
    __shared__ float prm[4];
    __shared__ int model;
    __shared__ float fb[3];
    if (threadIdx.x == 0) {
        bi = a.blk[blockIdx.x];
        s = a.sc[bi.scene];
        for (int i = 0; i < 4; ++i) prm[i] = a.params[bi.scene * 4 + i];
        model = a.models[bi.scene];
        const float* d = a.dforce + bi.scene * a.dforce_stride + (long long)(a.fo - 1) * 3;
        for (int c = 0; c < 3; ++c) fb[c] = d[c];
    }
    __syncthreads();
    constexpr bool WARP = VARIANT == P2G_WARP;
    long long p = bi.start + threadIdx.x;
    const bool active = p < bi.end;
    if (WARP && !active) p = bi.end - 1;  // the lane computes a copy and writes nothing
    float pg[4] = {0.f, 0.f, 0.f, 0.f};
    if (active || WARP) {
        const int kind = bi.kind;
        const bool liquid = kind == KIND_LIQUID;
        // ---- P2G adjoint of substep f
        float xb[3], vb[3], Cb[9];
        {
            float x[3];
            load3(a.cur, a.stride, OX, p, x);
            float m, mv[3], A[9];
            p2g_adj_affine<SVDJ>(a.cur, a.stride, s, prm, model, p, kind, m, mv, A);
            float Ab[9], vvb[3] = {0.f, 0.f, 0.f}, fxb[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int i = 0; i < 9; ++i) Ab[i] = 0.f;
            int base[3];
            float fx[3];
            if (locate(x, s.inv_dx, s.n, base, fx)) {
                float w[3][3], dw[3][3];
                bspline_d(fx, w, dw);
                p2g_adj_gather(a.pmb, s, base, fx, w, dw, m, mv, A, liquid, Ab, vvb, fxb);
            }
            float Fb[9];
            p2g_adj_core<SVDJ>(a, s, prm, model, p, kind, m, Ab, vvb, fxb, pg, xb, vb, Cb, Fb);
            if (active) {
                store9(a.adj_cur, a.stride, OF, p, Fb);
            } else {
#pragma unroll
                for (int i = 0; i < 4; ++i) pg[i] = 0.f;
            }
        }
        // ---- G2P adjoint of substep f-1 (g2p_adj_kernel) with the adjoint of state f
        float x[3];
        load3(a.cur2, a.stride, OX, p, x);
        float vnb[3], xbo[3] = {0.f, 0.f, 0.f};
        if (liquid) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                vnb[c] = vb[c] + s.dt * xb[c];
                xbo[c] = xb[c];
            }
        } else if (kind == KIND_ROD && s.rod_mode == DSTIR_ROD_PARTICLES) {
#pragma unroll
            for (int c = 0; c < 3; ++c) vnb[c] = -fb[c] * s.force_scale;
        } else {
            vnb[0] = vnb[1] = vnb[2] = 0.f;
        }
        int base[3];
        float fx[3];
        const bool in2 = locate(x, s.inv_dx, s.n, base, fx);
        const bool act2 = active && in2;
        if (WARP && !in2) {
            base[0] = base[1] = base[2] = 0;
            fx[0] = fx[1] = fx[2] = 1.f;
        }
        if (in2 || WARP) {
            float w[3][3], dw[3][3];
            bspline_d(fx, w, dw);
            // factored as in g2p_adj_kernel: vnb + c4 Cb (o - fx) = e + Cc o
            const float c4 = 4.f * s.inv_dx;
            float Cc[9], e[3];
#pragma unroll
            for (int q = 0; q < 9; ++q) Cc[q] = c4 * Cb[q];
#pragma unroll
            for (int q = 0; q < 3; ++q)
                e[q] = vnb[q] - (Cc[q * 3 + 0] * fx[0] + Cc[q * 3 + 1] * fx[1] + Cc[q * 3 + 2] * fx[2]);
            float fxb[3] = {0.f, 0.f, 0.f}, U[3] = {0.f, 0.f, 0.f};
            RunAgg ra;
            if (WARP) ra = run_agg_flags(act2 ? (base[0] * s.n + base[1]) * s.n + base[2] : run_agg_inactive_key());
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const int row = node_index(s, base[0] + i, base[1] + j, base[2]);
                    const float wij = w[i][0] * w[j][1], dxij = dw[i][0] * w[j][1], dyij = w[i][0] * dw[j][1];
                    float r[3];
#pragma unroll
                    for (int q = 0; q < 3; ++q) r[q] = e[q] + (float)i * Cc[q * 3 + 0] + (float)j * Cc[q * 3 + 1];
                    float4 cw[3];
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        const float W = wij * w[k][2];
                        const float rk0 = r[0] + (float)k * Cc[2], rk1 = r[1] + (float)k * Cc[5],
                                    rk2 = r[2] + (float)k * Cc[8];
                        float4* dst = a.ga + row + k;
                        const float g0 = W * rk0, g1 = W * rk1, g2 = W * rk2;
                        if (VARIANT == P2G_PLAIN) {
                            if (act2) {
                                float* dd = reinterpret_cast<float*>(dst);
                                atomicAdd(dd + 0, g0);
                                atomicAdd(dd + 1, g1);
                                atomicAdd(dd + 2, g2);
                            }
                        } else if (VARIANT == P2G_VEC) {
                            if (act2) red_add4(dst, g0, g1, g2, 0.f);
                        } else {
                            cw[k] = make_float4(g0, g1, g2, 0.f);
                        }
                        if (liquid) {
                            const float4 g = __ldg(a.vo2 + row + k);
                            const float Wb = g.x * rk0 + g.y * rk1 + g.z * rk2;
                            U[0] += W * g.x;
                            U[1] += W * g.y;
                            U[2] += W * g.z;
                            fxb[0] += Wb * dxij * w[k][2];
                            fxb[1] += Wb * dyij * w[k][2];
                            fxb[2] += Wb * wij * dw[k][2];
                        }
                    }
                    if (WARP) run_agg_scatter<3>(ra, a.ga + row, cw[0], cw[1], cw[2], act2);
                }
            if (liquid)
#pragma unroll
                for (int b = 0; b < 3; ++b)
                    xbo[b] += s.inv_dx * (fxb[b] - (Cc[0 * 3 + b] * U[0] + Cc[1 * 3 + b] * U[1] + Cc[2 * 3 + b] * U[2]));
        }
        if (liquid && active) store3(a.adj_prev, a.stride, OX, p, xbo);
    }
    if (bi.kind == KIND_LIQUID) {
        group_sum<4>(pg, sh, a.partial, a.counters + 2 * a.batch + bi.scene, blockIdx.x - bi.idx, bi.count,
                     a.pgrad + ((long long)a.fo * a.batch + bi.scene) * 4, 1.f, blockIdx.x);
    }
}

// ---------------------------------------------------------------------------
// layout and reduction helpers
// ---------------------------------------------------------------------------
__global__ void pack_state_kernel(const float* x, const float* v, const float* C, const float* F, float* st,
                                  long long stride, long long n) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= n) return;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        st[(OX + c) * stride + p] = x[p * 3 + c];
        st[(OV + c) * stride + p] = v ? v[p * 3 + c] : 0.f;
    }
#pragma unroll
    for (int c = 0; c < 9; ++c) {
        st[(OC + c) * stride + p] = C ? C[p * 9 + c] : 0.f;
        st[(OF + c) * stride + p] = F ? F[p * 9 + c] : ((c % 4 == 0) ? 1.f : 0.f);
    }
}

__global__ void unpack_state_kernel(const float* st, long long stride, long long n, float* x, float* v, float* C,
                                    float* F, const int* perm) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= n) return;
    long long q = perm ? (long long)perm[p] : p;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (x) x[q * 3 + c] = st[(OX + c) * stride + p];
        if (v) v[q * 3 + c] = st[(OV + c) * stride + p];
    }
#pragma unroll
    for (int c = 0; c < 9; ++c) {
        if (C) C[q * 9 + c] = st[(OC + c) * stride + p];
        if (F) F[q * 9 + c] = st[(OF + c) * stride + p];
    }
}

__global__ void iota_kernel(int* a, long long n) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p < n) a[p] = (int)p;
}

// out[b*4+c] = sum_t pgrad[(t*B+b)*4+c], one block per (b, c), fixed order
__global__ void reduce_pgrad_kernel(const float* pgrad, int T, int B, float* out) {
    __shared__ float sh[32][4];
    int b = blockIdx.x >> 2, c = blockIdx.x & 3;
    float acc[1] = {0.f};
    for (int t = threadIdx.x; t < T; t += blockDim.x) acc[0] += pgrad[((long long)t * B + b) * 4 + c];
    block_reduce<1>(acc, sh);
    if (threadIdx.x == 0) out[b * 4 + c] = acc[0];
}

// ---------------------------------------------------------------------------
// persistent segment kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_relaxed_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier of a cooperative launch (all blocks co-resident).  Thread
// 0 of each block publishes the block's writes (fence), arrives, and the last
// arrival opens the next generation with a release store; the others poll the
// generation with relaxed loads and, once it moved, take one acquire fence,
// which makes the other blocks' writes visible to the plain loads after the
// barrier.  The wait is bounded: past `limit_ns` the block raises
// DSTIR_STATUS_TIMEOUT and `abort`, and a block that sees `abort` stops
// waiting too.  Returns false, for the whole block, when the kernel must end.
// `expected`: arrivals that open the barrier (the grid's blocks, plus one in
// the test that makes every wait run out).
__device__ __forceinline__ bool grid_barrier(GridBar* b, unsigned expected, long long limit_ns, unsigned* status) {
    __shared__ int go;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned gen = ld_relaxed_gpu(&b->gen);
        __threadfence();
        const unsigned arrived = atomicAdd(&b->count, 1u) + 1u;
        if (arrived == expected) {
            b->count = 0u;  // ordered before the release of the next generation
            st_release_gpu(&b->gen, gen + 1u);
        } else {
            const unsigned long long t0 = global_ns();
            unsigned spins = 0;
            while (ld_relaxed_gpu(&b->gen) == gen) {
                if ((++spins & 63u) == 0u) {
                    if (ld_relaxed_gpu(&b->abort)) {
                        ok = 0;
                        break;
                    }
                    if ((long long)(global_ns() - t0) > limit_ns) {
                        atomicOr(status, DSTIR_STATUS_TIMEOUT);
                        atomicExch(&b->abort, 1u);
                        ok = 0;
                        break;
                    }
                }
            }
        }
        __threadfence();  // acquire: the writes released before the generation moved
        go = ok;
    }
    __syncthreads();
    return go != 0;
}

// A chain of forward substeps in one launch.  Per substep: P2G over the
// particle blocks, barrier, grid update over the node blocks and the rod-force
// blocks, barrier, G2P over the particle blocks.  Block b always takes the
// particle blocks b, b + gridDim.x, ..., so the state G2P writes is read by
// the same block's P2G of the next substep, and no barrier is needed between
// them; the grid update of the next substep comes after the next P2G
// barrier, by which time every block has finished its G2P reads of the
// velocity grid.  The P2G grid of each substep must start at zero (the grid
// update clears it with clear_pm, or the caller zeroed every slot).
template <bool SVDJ>
__global__ void __launch_bounds__(256, 2) seg_fwd_kernel(SegFwdArgs g) {
    const unsigned expected = gridDim.x + (unsigned)g.bar_extra;
    const int nvb_grid = g.a.n_gblocks + g.a.batch;
    for (int k = 0; k < g.nsteps; ++k) {
        FwdArgs a = g.a;
        a.cur = g.cur[k];
        a.next = g.next[k];
        a.pm = g.pm[k];
        a.vo = g.vo[k];
        a.box = g.box[k];
        a.f = g.f0 + k;
        a.fo = g.fo0 + k;
        for (int vb = blockIdx.x; vb < g.n_pblocks; vb += gridDim.x) {
            p2g_body<P2G_VEC, SVDJ, false>(a, vb);
            __syncthreads();
        }
        if (!grid_barrier(g.bar, expected, g.limit_ns, a.status)) return;
        for (int vb = blockIdx.x; vb < nvb_grid; vb += gridDim.x) {
            grid_body<true>(a, vb);
            __syncthreads();
        }
        if (!grid_barrier(g.bar, expected, g.limit_ns, a.status)) return;
        for (int vb = blockIdx.x; vb < g.n_pblocks; vb += gridDim.x) {
            g2p_body<false, false>(a, vb);
            __syncthreads();
        }
    }
}

// The reverse pass of up to kSegMax substeps (descending) in one launch.  Per
// substep: G2P adjoint (scatter into the grid adjoint), barrier, grid adjoint
// (clears the grid adjoint, writes the P/M adjoint), barrier, P2G adjoint
// (gathers the P/M adjoint).  As in seg_fwd_kernel a block keeps its particle
// blocks, so the state adjoint the P2G adjoint writes is read by the same
// block's G2P adjoint of the substep before; the next grid adjoint rewrites
// the P/M adjoint only after the next G2P-adjoint barrier, when every block
// has finished gathering it.
template <bool SVDJ>
__global__ void __launch_bounds__(256, 2) seg_adj_kernel(SegAdjArgs g) {
    const unsigned expected = gridDim.x + (unsigned)g.bar_extra;
    for (int q = 0; q < g.nsteps; ++q) {
        AdjArgs a = g.a;
        a.cur = g.cur[q];
        a.pm = g.pm[q];
        a.vo = g.vo[q];
        a.adj_next = g.adj_next[q];
        a.adj_cur = g.adj_cur[q];
        a.box = g.box[q];
        a.f = g.f0 - q;
        a.fo = g.fo0 - q;
        for (int vb = blockIdx.x; vb < g.n_pblocks; vb += gridDim.x) {
            g2p_adj_body<P2G_VEC, false>(a, vb);
            __syncthreads();
        }
        if (!grid_barrier(g.bar, expected, g.limit_ns, g.status)) return;
        for (int vb = blockIdx.x; vb < g.n_gblocks; vb += gridDim.x) {
            grid_adj_body<true>(a, vb);
            __syncthreads();
        }
        if (!grid_barrier(g.bar, expected, g.limit_ns, g.status)) return;
        for (int vb = blockIdx.x; vb < g.n_pblocks; vb += gridDim.x) {
            p2g_adj_body<SVDJ, false>(a, vb);
            __syncthreads();
        }
    }
}

int seg_max_blocks(bool svdj) {
    int dev = 0, sms = 0, coop = 0, f = 0, a = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return 0;
    if (svdj) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f, seg_fwd_kernel<true>, 256, 0) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, seg_adj_kernel<true>, 256, 0) != cudaSuccess)
            return 0;
    } else {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f, seg_fwd_kernel<false>, 256, 0) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, seg_adj_kernel<false>, 256, 0) != cudaSuccess)
            return 0;
    }
    return sms * (f < a ? f : a);
}

template <class Args>
cudaError_t coop_launch(void (*k)(Args), int grid, cudaStream_t st, const Args& g) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, g);
}

cudaError_t launch_seg_fwd(const SegFwdArgs& g, int grid, bool svdj, cudaStream_t st) {
    if (g.nsteps <= 0) return cudaSuccess;
    return svdj ? coop_launch(seg_fwd_kernel<true>, grid, st, g) : coop_launch(seg_fwd_kernel<false>, grid, st, g);
}
cudaError_t launch_seg_adj(const SegAdjArgs& g, int grid, bool svdj, cudaStream_t st) {
    if (g.nsteps <= 0) return cudaSuccess;
    return svdj ? coop_launch(seg_adj_kernel<true>, grid, st, g) : coop_launch(seg_adj_kernel<false>, grid, st, g);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
// Launch bounds.  MINB, the resident blocks per SM that the register
// allocation must allow, is set per kernel and per "tight" level: level 0
// keeps the allocation the compiler picks for 256-thread blocks (64 registers
// for P2G, 80 for G2P and the fused forward, about 110-130 for the
// adjoints); level 1 caps G2P and the fused forward at 64 and the adjoints at
// 80 registers (a few spilled bytes, half again as many resident warps);
// level 2 also caps P2G at 48; level 3 also caps the G2P adjoint at 64 (36
// spilled bytes; the P2G adjoint spills 340 bytes at 64 and stays at 80).
// Launch with programmatic stream serialisation when `pdl` is set (the
// kernels' pdl_enter keeps the ordering), else a plain launch.
// prio: a cudaLaunchAttributePriority value for this launch (0: none).
template <class Args>
void klaunch(void (*k)(Args), unsigned grid, unsigned block, cudaStream_t st, const Args& a, int prio = 0) {
    if (!a.pdl && !prio) {
        k<<<grid, block, 0, st>>>(a);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[2];
    unsigned na = 0;
    if (a.pdl) {
        at[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[na].val.programmaticStreamSerializationAllowed = 1;
        ++na;
    }
    if (prio) {
        at[na].id = cudaLaunchAttributePriority;
        at[na].val.priority = prio;
        ++na;
    }
    cfg.attrs = at;
    cfg.numAttrs = na;
    cudaLaunchKernelEx(&cfg, k, a);
}

void launch_p2g(const FwdArgs& a, int n_blocks, int block, int variant, bool svdj, cudaStream_t st, int tight) {
    if (n_blocks <= 0) return;
    const bool t2 = tight >= 2 && !svdj;
    void (*k)(FwdArgs);
    if (variant == P2G_PLAIN)
        k = svdj ? p2g_kernel<P2G_PLAIN, true, 4> : p2g_kernel<P2G_PLAIN, false, 4>;
    else if (variant == P2G_WARP)
        k = svdj ? p2g_kernel<P2G_WARP, true, 4> : t2 ? p2g_kernel<P2G_WARP, false, 5> : p2g_kernel<P2G_WARP, false, 4>;
    else
        k = svdj ? p2g_kernel<P2G_VEC, true, 4> : t2 ? p2g_kernel<P2G_VEC, false, 5> : p2g_kernel<P2G_VEC, false, 4>;
    klaunch(k, n_blocks, block, st, a);
}
void launch_grid(const FwdArgs& a, int n_gblocks, int gblock, cudaStream_t st) {
    if (n_gblocks <= 0) return;
    FwdArgs b = a;
    b.n_gblocks = n_gblocks;  // the last `batch` blocks compute the rod forces
    klaunch(grid_kernel, n_gblocks + a.batch, gblock, st, b, a.gprio);
}
void launch_g2p(const FwdArgs& a, int n_blocks, int block, cudaStream_t st, int tight, bool write_f) {
    if (n_blocks <= 0) return;
    void (*k)(FwdArgs) = write_f ? g2p_kernel<3, true> : tight >= 1 ? g2p_kernel<4, false> : g2p_kernel<3, false>;
    klaunch(k, n_blocks, block, st, a);
}
void launch_g2p_p2g(const FwdArgs& a, int n_blocks, int block, int variant, bool svdj, cudaStream_t st, int tight) {
    if (n_blocks <= 0) return;
    const bool t1 = tight >= 1;
    void (*k)(FwdArgs);
    if (variant == P2G_PLAIN)
        k = svdj ? g2p_p2g_kernel<P2G_PLAIN, true, 3> : g2p_p2g_kernel<P2G_PLAIN, false, 3>;
    else if (variant == P2G_WARP)
        k = svdj ? g2p_p2g_kernel<P2G_WARP, true, 3>
            : t1 ? g2p_p2g_kernel<P2G_WARP, false, 4>
                 : g2p_p2g_kernel<P2G_WARP, false, 3>;
    else
        k = svdj ? g2p_p2g_kernel<P2G_VEC, true, 3>
            : t1 ? g2p_p2g_kernel<P2G_VEC, false, 4>
                 : g2p_p2g_kernel<P2G_VEC, false, 3>;
    klaunch(k, n_blocks, block, st, a);
}
void launch_g2p_adj(const AdjArgs& a, int n_blocks, int block, int variant, cudaStream_t st, int tight) {
    if (n_blocks <= 0) return;
    const bool t1 = tight >= 1;
    void (*k)(AdjArgs);
    if (variant == P2G_PLAIN)
        k = g2p_adj_kernel<P2G_PLAIN, 2>;
    else if (variant == P2G_WARP)
        k = tight >= 3 ? g2p_adj_kernel<P2G_WARP, 4> : t1 ? g2p_adj_kernel<P2G_WARP, 3> : g2p_adj_kernel<P2G_WARP, 2>;
    else
        k = tight >= 3 ? g2p_adj_kernel<P2G_VEC, 4> : t1 ? g2p_adj_kernel<P2G_VEC, 3> : g2p_adj_kernel<P2G_VEC, 2>;
    klaunch(k, n_blocks, block, st, a);
}
void launch_grid_adj(const AdjArgs& a, int n_gblocks, int gblock, cudaStream_t st) {
    if (n_gblocks > 0) klaunch(grid_adj_kernel, n_gblocks, gblock, st, a, a.gprio);
}
void launch_p2g_adj(const AdjArgs& a, int n_blocks, int block, bool svdj, cudaStream_t st, int tight) {
    if (n_blocks <= 0) return;
    void (*k)(AdjArgs) = svdj ? p2g_adj_kernel<true, 2> : tight >= 1 ? p2g_adj_kernel<false, 3> : p2g_adj_kernel<false, 2>;
    klaunch(k, n_blocks, block, st, a);
}
void launch_p2g_adj_g2p_adj(const AdjArgs& a, int n_blocks, int block, int variant, bool svdj, cudaStream_t st,
                            int tight) {
    if (n_blocks <= 0) return;
    const bool t1 = tight >= 1;
    void (*k)(AdjArgs);
    if (variant == P2G_PLAIN)
        k = svdj ? p2g_adj_g2p_adj_kernel<P2G_PLAIN, true, 2> : p2g_adj_g2p_adj_kernel<P2G_PLAIN, false, 2>;
    else if (variant == P2G_WARP)
        k = svdj ? p2g_adj_g2p_adj_kernel<P2G_WARP, true, 2>
            : t1 ? p2g_adj_g2p_adj_kernel<P2G_WARP, false, 3>
                 : p2g_adj_g2p_adj_kernel<P2G_WARP, false, 2>;
    else
        k = svdj ? p2g_adj_g2p_adj_kernel<P2G_VEC, true, 2>
            : t1 ? p2g_adj_g2p_adj_kernel<P2G_VEC, false, 3>
                 : p2g_adj_g2p_adj_kernel<P2G_VEC, false, 2>;
    klaunch(k, n_blocks, block, st, a);
}
void launch_pack_state(const float* x, const float* v, const float* C, const float* F, float* st,
                       long long stride, long long n, cudaStream_t s) {
    if (n > 0) pack_state_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, v, C, F, st, stride, n);
}
void launch_iota(int* a, long long n, cudaStream_t s) {
    if (n > 0) iota_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, n);
}
void launch_unpack_state(const float* st, long long stride, long long n, float* x, float* v, float* C,
                         float* F, const int* perm, cudaStream_t s) {
    if (n > 0) unpack_state_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(st, stride, n, x, v, C, F, perm);
}
void launch_reduce_pgrad(const float* pgrad, int T, int B, float* out, cudaStream_t s) {
    if (B > 0) reduce_pgrad_kernel<<<B * 4, 256, 0, s>>>(pgrad, T, B, out);
}

}  // namespace dstir
