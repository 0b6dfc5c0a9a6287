// Per-particle pieces of the P2G adjoint (the reverse of p2g,
// simulation_functions.py:104-196, and of compute_F_tmp :39-42) shared by the
// per-particle kernel (kernels.cu) and the brick kernel (binning.cu).  The work
// is split so that few values stay live across the 27-node gather:
//   p2g_adj_affine   recompute the particle's affine momentum A and m v'
//   (caller)         gather the P/M adjoint over the stencil -> Ab, vvb, fxb
//   p2g_adj_finish   reload C and F; stress, bulk, viscosity and F_tmp
//                    adjoints; write the state adjoint; parameter partials
#pragma once

#include "common.cuh"
#include "device_util.cuh"
#include "internal.h"
#include "svd.cuh"

namespace dstir {

// NC: load policy of the state reads (see ldp in device_util.cuh).
template <bool SVDJ, bool NC = true>
__device__ __forceinline__ void p2g_adj_affine(const float* cur, long long stride, const SceneDev& s,
                                               const float* prm, int model, long long p, int kind, float& m,
                                               float mv[3], float A[9]) {
    float v[3], C[9];
    load3<NC>(cur, stride, OV, p, v);
    load9<NC>(cur, stride, OC, p, C);
    if (kind == KIND_LIQUID) {
        float F[9];
        load9<NC>(cur, stride, OF, p, F);
        LiquidP2G q;
        liquid_p2g<SVDJ>(s, model, prm, v, C, F, q);
        m = s.m_liq;
#pragma unroll
        for (int i = 0; i < 9; ++i) A[i] = q.A[i];
#pragma unroll
        for (int c = 0; c < 3; ++c) mv[c] = m * q.vv[c];
    } else {
        m = (kind == KIND_ROD) ? s.m_rod : s.m_cont;
#pragma unroll
        for (int i = 0; i < 9; ++i) A[i] = m * C[i];
#pragma unroll
        for (int c = 0; c < 3; ++c) mv[c] = m * v[c];
    }
}

// Gather contribution of one stencil node (weight W, derivative weights
// dWx/dWy/dWz in fx, dpos dp, node adjoint gb) to Ab, vvb (not yet times m)
// and fxb.
__device__ __forceinline__ void p2g_adj_node(float W, float dWx, float dWy, float dWz, const float dp[3], float4 gb,
                                             float m, const float mv[3], const float A[9], float dx, bool liquid,
                                             float Ab[9], float vvb[3], float fxb[3]) {
    float gbv[3] = {gb.x, gb.y, gb.z};
    float Wb = gb.w * m;
#pragma unroll
    for (int aa = 0; aa < 3; ++aa) {
        float ad = A[aa * 3 + 0] * dp[0] + A[aa * 3 + 1] * dp[1] + A[aa * 3 + 2] * dp[2];
        Wb += gbv[aa] * (mv[aa] + ad);
        vvb[aa] += W * gbv[aa];
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) Ab[aa * 3 + bb] += W * gbv[aa] * dp[bb];
    }
    if (liquid) {
#pragma unroll
        for (int bb = 0; bb < 3; ++bb)
            fxb[bb] -= W * dx * (A[0 * 3 + bb] * gbv[0] + A[1 * 3 + bb] * gbv[1] + A[2 * 3 + bb] * gbv[2]);
        fxb[0] += Wb * dWx;
        fxb[1] += Wb * dWy;
        fxb[2] += Wb * dWz;
    }
}

// The same 27-node gather in factored form.  With dp = (o - fx) dx for node
// offset o = (i, j, k):
//   A dp + m v'         = c + dx (i A_0 + j A_1 + k A_2),   c = m v' - dx A fx
//   Ab = sum W g dp^T   = dx (T - S fx^T),  S = sum W g,  T = sum W g o^T
//   fxb -= dx sum W A^T g  ->  -dx A^T S, once after the loop,
// so a node costs its weight products, one float4 load, a 4-term dot product
// for Wb and a handful of adds, instead of the three 3x3 products of
// p2g_adj_node.  `pmb` is the P/M-adjoint grid, `row0` the node index of the
// stencil base (k innermost).  NC: load policy of the pmb reads.
template <bool NC = true>
__device__ __forceinline__ void p2g_adj_gather(const float4* pmb, const SceneDev& s,
                                               const int base[3], const float fx[3], const float w[3][3],
                                               const float dw[3][3], float m, const float mv[3],
                                               const float A[9], bool liquid, float Ab[9], float vvb[3],
                                               float fxb[3]) {
    const float dx = s.dx;
    float c[3], Ad[9];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        c[a] = mv[a] - dx * (A[a * 3 + 0] * fx[0] + A[a * 3 + 1] * fx[1] + A[a * 3 + 2] * fx[2]);
#pragma unroll
        for (int b = 0; b < 3; ++b) Ad[a * 3 + b] = dx * A[a * 3 + b];
    }
    float S[3] = {0.f, 0.f, 0.f}, T[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) T[q] = 0.f;
    float fb[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const float4* rowp = pmb + node_index(s, base[0] + i, base[1] + j, base[2]);
            const float wij = w[i][0] * w[j][1], dxij = dw[i][0] * w[j][1], dyij = w[i][0] * dw[j][1];
            float r[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) r[a] = c[a] + (float)i * Ad[a * 3 + 0] + (float)j * Ad[a * 3 + 1];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float4 g = ldp<NC>(rowp + k);
                const float W = wij * w[k][2];
                const float rk0 = r[0] + (float)k * Ad[2], rk1 = r[1] + (float)k * Ad[5], rk2 = r[2] + (float)k * Ad[8];
                const float Wb = g.w * m + g.x * rk0 + g.y * rk1 + g.z * rk2;
                const float wg[3] = {W * g.x, W * g.y, W * g.z};
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    S[a] += wg[a];
                    if (i) T[a * 3 + 0] += (float)i * wg[a];
                    if (j) T[a * 3 + 1] += (float)j * wg[a];
                    if (k) T[a * 3 + 2] += (float)k * wg[a];
                }
                if (liquid) {
                    fb[0] += Wb * dxij * w[k][2];
                    fb[1] += Wb * dyij * w[k][2];
                    fb[2] += Wb * wij * dw[k][2];
                }
            }
        }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        vvb[a] = S[a];
#pragma unroll
        for (int b = 0; b < 3; ++b) Ab[a * 3 + b] = dx * (T[a * 3 + b] - fx[b] * S[a]);
    }
    if (liquid) {
#pragma unroll
        for (int b = 0; b < 3; ++b)
            fxb[b] = fb[b] - (Ad[0 * 3 + b] * S[0] + Ad[1 * 3 + b] * S[1] + Ad[2 * 3 + b] * S[2]);
    } else {
        fxb[0] = fxb[1] = fxb[2] = 0.f;
    }
}

// The adjoint of the state at substep f (xb, vb, Cb, Fb) from the stencil
// gather results; parameter partials are added to pg.
template <bool SVDJ, bool NC = true>
__device__ __forceinline__ void p2g_adj_core(const AdjArgs& a, const SceneDev& s, const float* prm, int model,
                                             long long p, int kind, float m, const float Ab[9], const float vvb[3],
                                             const float fxb[3], float pg[4], float xb[3], float vb[3], float Cb[9],
                                             float Fb[9]) {
#pragma unroll
    for (int c = 0; c < 3; ++c) vb[c] = vvb[c] * m;
    if (kind != KIND_LIQUID) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            Cb[i] = m * Ab[i];
            Fb[i] = 0.f;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) xb[c] = vb[c] = 0.f;
        return;
    }
    load3<NC>(a.adj_cur, a.stride, OX, p, xb);  // G2P part, written by the G2P adjoint
#pragma unroll
    for (int c = 0; c < 3; ++c) xb[c] += s.inv_dx * fxb[c];
    float C[9], F[9], IC[9], Ft[9];
    load9<NC>(a.cur, a.stride, OC, p, C);
    load9<NC>(a.cur, a.stride, OF, p, F);
#pragma unroll
    for (int i = 0; i < 9; ++i) IC[i] = s.dt * C[i] + ((i % 4 == 0) ? 1.f : 0.f);
    matmul3(IC, F, Ft);
    float U[9], sg[3], Vm[9], J;
    if (SVDJ && s.j_mode == DSTIR_J_SVD) {
        svd3(Ft, U, sg, Vm);
        J = sg[0] * sg[1] * sg[2];
    } else {
        J = det3(Ft);
    }
    float nrm2 = 0.f;
#pragma unroll
    for (int i = 0; i < 9; ++i) nrm2 += C[i] * C[i];
    float nrm = sqrtf(nrm2);
    Visc vs = viscosity<true>(model, prm, nrm + 1e-6f);
    float sigb[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        Cb[i] = m * Ab[i];
        sigb[i] = s.alpha * Ab[i];
    }
    float etab = 0.f;
#pragma unroll
    for (int aa = 0; aa < 3; ++aa)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) {
            float Dab = 0.5f * (C[aa * 3 + bb] + C[bb * 3 + aa]);
            etab += sigb[aa * 3 + bb] * Dab;
            Cb[aa * 3 + bb] += vs.eta * 0.5f * (sigb[aa * 3 + bb] + sigb[bb * 3 + aa]);
        }
    float trb = sigb[0] + sigb[4] + sigb[8];
    float Jb = trb * (s.bulk / 2.f) * (2.f * J - 1.f);
    float Ftb[9];
    load9<NC>(a.adj_next, a.stride, OF, p, Ftb);  // F[f+1] = F_tmp
    if (SVDJ && s.j_mode == DSTIR_J_SVD) {
        float gS[3] = {Jb * sg[1] * sg[2], Jb * sg[0] * sg[2], Jb * sg[0] * sg[1]};
        float z[9], gA[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) z[i] = 0.f;
        svd3_backward(z, gS, z, U, sg, Vm, gA);
#pragma unroll
        for (int i = 0; i < 9; ++i) Ftb[i] += gA[i];
    } else {
        float cf[9];
        cof3(Ft, cf);
#pragma unroll
        for (int i = 0; i < 9; ++i) Ftb[i] += Jb * cf[i];
    }
    float gammab = etab * vs.deta_dgamma;
#pragma unroll
    for (int i = 0; i < 4; ++i) pg[i] += etab * vs.dp[i];
    if (nrm > 0.f) {
        float inv = gammab / nrm;
#pragma unroll
        for (int i = 0; i < 9; ++i) Cb[i] += inv * C[i];
    }
#pragma unroll
    for (int aa = 0; aa < 3; ++aa)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) {
            float sF = 0.f, sC = 0.f;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                sF += IC[c * 3 + aa] * Ftb[c * 3 + bb];
                sC += Ftb[aa * 3 + c] * F[bb * 3 + c];
            }
            Fb[aa * 3 + bb] = sF;
            Cb[aa * 3 + bb] += s.dt * sC;
        }
}

// p2g_adj_core followed by storing the whole state adjoint into a.adj_cur.
template <bool SVDJ, bool NC = true>
__device__ __forceinline__ void p2g_adj_finish(const AdjArgs& a, const SceneDev& s, const float* prm, int model,
                                               long long p, int kind, float m, const float Ab[9], float vvb[3],
                                               const float fxb[3], float pg[4]) {
    float xb[3], vb[3], Cb[9], Fb[9];
    p2g_adj_core<SVDJ, NC>(a, s, prm, model, p, kind, m, Ab, vvb, fxb, pg, xb, vb, Cb, Fb);
    store3(a.adj_cur, a.stride, OX, p, xb);
    store3(a.adj_cur, a.stride, OV, p, vb);
    store9(a.adj_cur, a.stride, OC, p, Cb);
    store9(a.adj_cur, a.stride, OF, p, Fb);
}

}  // namespace dstir
