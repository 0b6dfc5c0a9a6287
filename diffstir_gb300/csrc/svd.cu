// Batched 3x3 SVD and SVD-backward kernels behind dstir_svd3 /
// dstir_svd3_backward (the reference's svd :55-58 and svd_grad :90-93 of
// src/simulator/simulation_functions.py, which act on F_tmp per particle).
#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"
#include "svd.cuh"

namespace dstir {

__global__ void svd3_kernel(const float* A, float* U, float* S, float* V, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float a[9], u[9], s[3], v[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) a[c] = A[i * 9 + c];
    svd3(a, u, s, v);
#pragma unroll
    for (int c = 0; c < 9; ++c) {
        U[i * 9 + c] = u[c];
        V[i * 9 + c] = v[c];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) S[i * 3 + c] = s[c];
}

__global__ void svd3_backward_kernel(const float* gU, const float* gS, const float* gV, const float* U,
                                     const float* S, const float* V, float* gA, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float a[9], b[3], c[9], u[9], s[3], v[9], o[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        a[k] = gU[i * 9 + k];
        c[k] = gV[i * 9 + k];
        u[k] = U[i * 9 + k];
        v[k] = V[i * 9 + k];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        b[k] = gS[i * 3 + k];
        s[k] = S[i * 3 + k];
    }
    svd3_backward(a, b, c, u, s, v, o);
#pragma unroll
    for (int k = 0; k < 9; ++k) gA[i * 9 + k] = o[k];
}

void launch_svd3(const float* A, float* U, float* S, float* V, long long n, cudaStream_t s) {
    if (n > 0) svd3_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(A, U, S, V, n);
}

void launch_svd3_backward(const float* gU, const float* gS, const float* gV, const float* U, const float* S,
                          const float* V, float* gA, long long n, cudaStream_t s) {
    if (n > 0) svd3_backward_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(gU, gS, gV, U, S, V, gA, n);
}

}  // namespace dstir
