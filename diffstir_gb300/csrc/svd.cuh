// Per-thread 3x3 singular value decomposition and its backward pass.
//
// Forward: cyclic Jacobi eigen-decomposition of A^T A (exact rotation angles,
// fixed sweep cap) gives V and the squared singular values; A V is then
// reduced to upper-triangular form by three Givens rotations, whose product
// is U.  This is the structure of McAdams, Selle, Tamstorf, Teran and Sifakis,
// "Computing the Singular Value Decomposition of 3x3 matrices with minimal
// branching and elementary floating point operations" (UW-Madison TR1690,
// 2011), with exact instead of approximate Givens angles.  Convention (the
// one of the reference's ti.svd, simulation_functions.py:58): det U = det V =
// +1, s0 >= s1 >= |s2|, and s2 carries the sign of det A.
//
// Backward: backward_svd of simulation_functions.py:61-87 (clamp :61-67).  The
// f_ij = 1/clamp(s_j^2 - s_i^2) factors and the skew terms they multiply are
// evaluated in FP64, because they blow up as singular values meet; the rest
// is FP32.
#pragma once

#include <cuda_runtime.h>

namespace dstir {

__device__ __forceinline__ void jacobi_rotate(float* S, float* V, int p, int q) {
    float apq = S[p * 3 + q];
    if (apq == 0.f) return;
    float app = S[p * 3 + p], aqq = S[q * 3 + q];
    float theta = (aqq - app) / (2.f * apq);
    float t = copysignf(1.f, theta) / (fabsf(theta) + sqrtf(theta * theta + 1.f));
    float c = rsqrtf(t * t + 1.f), s = t * c;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float skp = S[k * 3 + p], skq = S[k * 3 + q];
        S[k * 3 + p] = c * skp - s * skq;
        S[k * 3 + q] = s * skp + c * skq;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float spk = S[p * 3 + k], sqk = S[q * 3 + k];
        S[p * 3 + k] = c * spk - s * sqk;
        S[q * 3 + k] = s * spk + c * sqk;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float vkp = V[k * 3 + p], vkq = V[k * 3 + q];
        V[k * 3 + p] = c * vkp - s * vkq;
        V[k * 3 + q] = s * vkp + c * vkq;
    }
}

__device__ __forceinline__ void swap_cols(float* V, float* ev, int a, int b) {
    float t = ev[a];
    ev[a] = ev[b];
    ev[b] = t;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float x = V[r * 3 + a];
        V[r * 3 + a] = V[r * 3 + b];
        V[r * 3 + b] = -x;  // keeps det V = +1
    }
}

__device__ __forceinline__ void givens_qr(float* B, float* Q, int r1, int r2, int col) {
    float a = B[r1 * 3 + col], b = B[r2 * 3 + col];
    float rr = sqrtf(a * a + b * b);
    float c = 1.f, s = 0.f;
    if (rr > 0.f) {
        float inv = 1.f / rr;
        c = a * inv;
        s = b * inv;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float x1 = B[r1 * 3 + k], x2 = B[r2 * 3 + k];
        B[r1 * 3 + k] = c * x1 + s * x2;
        B[r2 * 3 + k] = -s * x1 + c * x2;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float q1 = Q[k * 3 + r1], q2 = Q[k * 3 + r2];
        Q[k * 3 + r1] = c * q1 + s * q2;
        Q[k * 3 + r2] = -s * q1 + c * q2;
    }
}

__device__ __forceinline__ void svd3(const float* A, float* U, float* sg, float* V) {
    float S[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            S[i * 3 + j] = A[0 * 3 + i] * A[0 * 3 + j] + A[1 * 3 + i] * A[1 * 3 + j] + A[2 * 3 + i] * A[2 * 3 + j];
#pragma unroll
    for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.f : 0.f;
    for (int sweep = 0; sweep < 8; ++sweep) {
        float off = S[1] * S[1] + S[2] * S[2] + S[5] * S[5];
        float dg = S[0] * S[0] + S[4] * S[4] + S[8] * S[8];
        if (!(off > 1e-14f * dg)) break;
        jacobi_rotate(S, V, 0, 1);
        jacobi_rotate(S, V, 0, 2);
        jacobi_rotate(S, V, 1, 2);
    }
    float ev[3] = {S[0], S[4], S[8]};
    // sort descending (sorting network of 3), swaps keep det V = +1
    if (ev[0] < ev[1]) swap_cols(V, ev, 0, 1);
    if (ev[0] < ev[2]) swap_cols(V, ev, 0, 2);
    if (ev[1] < ev[2]) swap_cols(V, ev, 1, 2);
    float B[9];
    matmul3(A, V, B);
    float Q[9] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f};
    givens_qr(B, Q, 0, 1, 0);
    givens_qr(B, Q, 0, 2, 0);
    givens_qr(B, Q, 1, 2, 1);
#pragma unroll
    for (int i = 0; i < 9; ++i) U[i] = Q[i];
    sg[0] = B[0];
    sg[1] = B[4];
    sg[2] = B[8];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        if (sg[i] < 0.f) {
            sg[i] = -sg[i];
            sg[2] = -sg[2];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                U[r * 3 + i] = -U[r * 3 + i];
                U[r * 3 + 2] = -U[r * 3 + 2];
            }
        }
    }
}

__device__ __forceinline__ double clamp_gap(double a) { return a >= 0.0 ? fmax(a, 1e-6) : fmin(a, -1e-6); }

// gA = u_term + v_term + U diag(gs) V^T  (simulation_functions.py:72-87)
__device__ __forceinline__ void svd3_backward(const float* gU, const float* gs, const float* gV, const float* U,
                                              const float* sg, const float* V, float* gA) {
    double s2[3] = {(double)sg[0] * sg[0], (double)sg[1] * sg[1], (double)sg[2] * sg[2]};
    double f[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) f[i * 3 + j] = (i == j) ? 0.0 : 1.0 / clamp_gap(s2[j] - s2[i]);
    // skew parts K_u = f * (U^T gU - gU^T U), K_v = f * (V^T gV - gV^T V)
    float Ku[9], Kv[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double a = 0.0, b = 0.0, c = 0.0, d = 0.0;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                a += (double)U[k * 3 + i] * gU[k * 3 + j];
                b += (double)gU[k * 3 + i] * U[k * 3 + j];
                c += (double)V[k * 3 + i] * gV[k * 3 + j];
                d += (double)gV[k * 3 + i] * V[k * 3 + j];
            }
            Ku[i * 3 + j] = (float)(f[i * 3 + j] * (a - b));
            Kv[i * 3 + j] = (float)(f[i * 3 + j] * (c - d));
        }
    // inner = (Ku S) + (S Kv) ; gA = U (inner + diag(gs)) V^T
    float M[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            M[i * 3 + j] = Ku[i * 3 + j] * sg[j] + sg[i] * Kv[i * 3 + j] + ((i == j) ? gs[i] : 0.f);
    float T1[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            T1[i * 3 + j] = M[i * 3 + 0] * V[j * 3 + 0] + M[i * 3 + 1] * V[j * 3 + 1] + M[i * 3 + 2] * V[j * 3 + 2];
    matmul3(U, T1, gA);
}

}  // namespace dstir
