// Device helpers shared by the particle kernels (kernels.cu) and the binned
// kernels (binning.cu): deterministic block/group reductions, vector atomics,
// SoA state loads, and the liquid stress of P2G (simulation_functions.py:111-152).
#pragma once

#include <cuda_runtime.h>

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
// result does not depend on scheduling) and writes it to out[0..NV).
template <int NV>
__device__ __forceinline__ void group_sum(float (&v)[NV], float (*sh)[4], float* partial, unsigned* counter,
                                          int group_first, int group_count, float* out, float scale) {
    __shared__ bool is_last;
    block_reduce<NV>(v, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) partial[(long long)blockIdx.x * 4 + c] = v[c];
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

__device__ __forceinline__ void red_add4(float4* p, float a, float b, float c, float d) {
    atomicAdd(p, make_float4(a, b, c, d));
}

// ---------------------------------------------------------------------------
// state loads
// ---------------------------------------------------------------------------
__device__ __forceinline__ void load3(const float* st, long long stride, int o, long long p, float* v) {
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = __ldg(st + (long long)(o + c) * stride + p);
}
__device__ __forceinline__ void load9(const float* st, long long stride, int o, long long p, float* v) {
#pragma unroll
    for (int c = 0; c < 9; ++c) v[c] = __ldg(st + (long long)(o + c) * stride + p);
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
