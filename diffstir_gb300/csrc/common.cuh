// Device-side data layout and per-particle math shared by the forward and
// adjoint kernels of the MLS-MPM stirring path (sm_103a).
//
// Reference: src/simulator/simulation_functions.py (Taichi).  Every formula
// here restates one of its lines; the line is cited where it is used.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/diffstir.h"

namespace dstir {

// Particle state, structure of arrays: component c of particle p lives at
// st[c * stride + p]; 24 components x3 v3 C9 F9 (C, F row-major).
constexpr int NS = 24;
constexpr int OX = 0, OV = 3, OC = 6, OF = 15;

enum Kind { KIND_LIQUID = 0, KIND_ROD = 1, KIND_CONTAINER = 2 };

// Per-scene constants in device memory (derived from DstirSceneDesc).
struct SceneDev {
    int n, bound, rod_mode, j_mode, container_wall, model;
    int n_liquid, n_rod, n_container;
    int nbr;          // bricks of 4x4x4 cells per axis, ceil(n/4)
    long long p0;     // first particle (global index) of the scene
    long long goff;   // first grid node of the scene
    long long koff;   // first brick-major bin key of the scene (64 keys per brick)
    float dt, dx, inv_dx, gravity, bulk, alpha;  // alpha = -dt*V_p*4*inv_dx^2 (:150)
    float m_liq, m_rod, m_cont, force_scale;
    float ccx, ccz, cr2;  // container axis and squared projection radius (:205-207)
    float rod_r2;         // cylinder rod: squared radius
};

// One CUDA block of a particle kernel covers particles [start, end) of a single
// (scene, kind); `idx` is its rank among the `count` blocks of that pair, so
// block reductions can be finished deterministically by the last block.
struct BlockInfo {
    int scene, kind, idx, count;
    long long start, end;
};

// One CUDA block of a grid kernel covers nodes [start, end) of one scene.
struct GridBlock {
    int scene, idx, count, pad;
    long long start, end;
};

// (i, j, k) of a scene-local node index (k innermost) in 32-bit arithmetic;
// n <= 1024, so local < 2^30
__device__ __forceinline__ void node_ijk(int local, int n, int& i, int& j, int& k) {
    const int nn = n * n;
    i = local / nn;
    const int r = local - i * nn;
    j = r / n;
    k = r - j * n;
}

// Block-cooperative copy of a scene descriptor into shared memory (one word
// per thread of the first warp instead of a serial struct copy by thread 0).
// Call from every thread of the block; a __syncthreads() must follow.
__device__ __forceinline__ void load_scene_shared(SceneDev& dst, const SceneDev* src) {
    static_assert(sizeof(SceneDev) % 4 == 0 && sizeof(SceneDev) / 4 <= 32, "SceneDev copy");
    const int words = (int)(sizeof(SceneDev) / 4);
    if (threadIdx.x < words)
        reinterpret_cast<int*>(&dst)[threadIdx.x] = __ldg(reinterpret_cast<const int*>(src) + threadIdx.x);
}

__device__ __forceinline__ float* comp(float* st, long long stride, int c) { return st + (long long)c * stride; }
__device__ __forceinline__ const float* comp(const float* st, long long stride, int c) {
    return st + (long long)c * stride;
}

// base / fx of simulation_functions.py:106-107 (truncating int cast)
__device__ __forceinline__ bool locate(const float x[3], float inv_dx, int n, int base[3], float fx[3]) {
    bool ok = true;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float X = x[c] * inv_dx;
        base[c] = (int)(X - 0.5f);
        fx[c] = X - (float)base[c];
        ok = ok && base[c] >= 0 && base[c] <= n - 3;
    }
    return ok;
}

// quadratic B-spline weights (:108-110) and their derivatives in fx
__device__ __forceinline__ void bspline(const float fx[3], float w[3][3]) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float t0 = 1.5f - fx[d], t1 = fx[d] - 1.0f, t2 = fx[d] - 0.5f;
        w[0][d] = 0.5f * t0 * t0;
        w[1][d] = 0.75f - t1 * t1;
        w[2][d] = 0.5f * t2 * t2;
    }
}

__device__ __forceinline__ void bspline_d(const float fx[3], float w[3][3], float dw[3][3]) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float t0 = 1.5f - fx[d], t1 = fx[d] - 1.0f, t2 = fx[d] - 0.5f;
        w[0][d] = 0.5f * t0 * t0;
        w[1][d] = 0.75f - t1 * t1;
        w[2][d] = 0.5f * t2 * t2;
        dw[0][d] = -t0;
        dw[1][d] = -2.0f * t1;
        dw[2][d] = t2;
    }
}

// 32-bit: dstir_create refuses batches whose nodes together exceed INT_MAX.
__device__ __forceinline__ int node_index(const SceneDev& s, int i, int j, int k) {
    return (int)s.goff + (i * s.n + j) * s.n + k;
}
// The same index in 64-bit arithmetic: the form G2P's gathers schedule best
// with (measured: G2P 4% shorter with it, the P2G adjoint 3% longer).
__device__ __forceinline__ long long node_index64(const SceneDev& s, int i, int j, int k) {
    return s.goff + ((long long)i * s.n + j) * s.n + k;
}

// Brick-major bin key of cell (i,j,k): bricks of 4x4x4 cells in (i,j,k)-major
// order, then the cell inside its brick, so that the 64 cells of a brick own
// one contiguous range of the sorted particle list.
__device__ __forceinline__ long long brick_key(const SceneDev& s, int i, int j, int k) {
    long long br = ((long long)(i >> 2) * s.nbr + (j >> 2)) * s.nbr + (k >> 2);
    return s.koff + br * 64 + (((i & 3) * 4 + (j & 3)) * 4 + (k & 3));
}

// One CTA of a brick kernel: the brick's first cell and its first bin key.
struct BrickInfo {
    int scene, bi, bj, bk;
    long long key0;
    int idx, count;  // rank of the brick among the scene's bricks, and their number
};

__device__ __forceinline__ void matmul3(const float* A, const float* B, float* o) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            o[i * 3 + j] = A[i * 3 + 0] * B[0 * 3 + j] + A[i * 3 + 1] * B[1 * 3 + j] + A[i * 3 + 2] * B[2 * 3 + j];
}

__device__ __forceinline__ float det3(const float* a) {
    return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
           a[2] * (a[3] * a[7] - a[4] * a[6]);
}

__device__ __forceinline__ void cof3(const float* a, float* c) {
    c[0] = a[4] * a[8] - a[5] * a[7];
    c[1] = -(a[3] * a[8] - a[5] * a[6]);
    c[2] = a[3] * a[7] - a[4] * a[6];
    c[3] = -(a[1] * a[8] - a[2] * a[7]);
    c[4] = a[0] * a[8] - a[2] * a[6];
    c[5] = -(a[0] * a[7] - a[1] * a[6]);
    c[6] = a[1] * a[5] - a[2] * a[4];
    c[7] = -(a[0] * a[5] - a[2] * a[3]);
    c[8] = a[0] * a[4] - a[1] * a[3];
}

// Viscosity models (:118-146) with partials in gamma and in the 4 parameters.
struct Visc {
    float eta, deta_dgamma;
    float dp[4];
};

template <bool WANT_GRAD>
__device__ __forceinline__ Visc viscosity(int model, const float* prm, float gamma) {
    Visc o;
    o.deta_dgamma = 0.f;
    o.dp[0] = o.dp[1] = o.dp[2] = o.dp[3] = 0.f;
    if (model == DSTIR_MODEL_CARREAU) {
        float eta0 = prm[0], einf = prm[1], n = prm[2], lam = prm[3];
        float lg = lam * gamma;
        float B = 1.f + lg * lg;
        float e = (n - 1.f) / 2.f;
        float Be = powf(B, e);
        o.eta = einf + (eta0 - einf) * Be;
        if (WANT_GRAD) {
            float dBe = e * powf(B, e - 1.f);
            o.dp[0] = Be;
            o.dp[1] = 1.f - Be;
            o.dp[2] = (eta0 - einf) * Be * logf(B) * 0.5f;
            o.dp[3] = (eta0 - einf) * dBe * 2.f * lg * gamma;
            o.deta_dgamma = (eta0 - einf) * dBe * 2.f * lg * lam;
        }
    } else if (model == DSTIR_MODEL_CROSS) {
        float eta0 = prm[0], einf = prm[1], n = prm[2], lam = prm[3];
        float lg = lam * gamma;
        float q = powf(lg, n - 1.f);
        float inv = 1.f / (1.f + q);
        o.eta = einf + (eta0 - einf) * inv;
        if (WANT_GRAD) {
            float deta_dq = -(eta0 - einf) * inv * inv;
            float dq = (n - 1.f) * powf(lg, n - 2.f);
            o.dp[0] = inv;
            o.dp[1] = 1.f - inv;
            o.dp[2] = deta_dq * q * logf(lg);
            o.dp[3] = deta_dq * dq * gamma;
            o.deta_dgamma = deta_dq * dq * lam;
        }
    } else {  // Herschel-Bulkley, power law when tau_y = 0
        float K = prm[0], tau = prm[1], n = prm[2];
        float gp = powf(gamma, n - 1.f);
        float delta = K * gp;
        o.eta = tau / gamma;
        if (WANT_GRAD) {
            o.deta_dgamma = -tau / (gamma * gamma);
            o.dp[1] = 1.f / gamma;
        }
        if (delta > 0.f) {
            o.eta += delta;
            if (WANT_GRAD) {
                o.dp[0] = gp;
                o.dp[2] = delta * logf(gamma);
                o.deta_dgamma += K * (n - 1.f) * powf(gamma, n - 2.f);
            }
        }
    }
    return o;
}

}  // namespace dstir
