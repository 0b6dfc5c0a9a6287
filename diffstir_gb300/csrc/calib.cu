// Throughput probes for the rooflines of the particle kernels, measured on
// the GPU at hand.  dstir_measure_red_rate: L2 vector reductions
// (red.global.add.v4.f32), the operation that bounds the warp-aggregated P2G
// scatter and the G2P-adjoint scatter.  dstir_measure_fp32_rate: FP32 FMA
// throughput, the denominator of the kernels' FP32 fraction.
//
// RED probe: every warp issues `reps` vector REDs; lane l of a warp adds to node
// row + l of a float4 grid of n_nodes nodes, with row a pseudo-random multiple
// of 32 per (warp, rep).  One instruction therefore covers 32 consecutive
// 16-byte nodes, 16 sectors of 32 bytes, the best case of the scatter kernels
// (a warp on 32 consecutive cells of one grid row).  The grid is sized like a
// 64^3 scene (4 MB), so it stays in L2 and the REDs, not DRAM, set the rate.
#include <cuda_runtime.h>

#include "../../include/diffstir.h"

namespace {

__global__ void __launch_bounds__(256) red_probe_kernel(float4* grid, long long rows, int reps) {
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    unsigned h = warp * 2654435761u + 12345u;
    for (int r = 0; r < reps; ++r) {
        h = h * 1664525u + 1013904223u;  // LCG step, identical in every lane
        const long long row = (long long)(h % (unsigned)rows) * 32;
        atomicAdd(grid + row + lane, make_float4(1.f, 1.f, 1.f, 1.f));
    }
}

// Eight independent FMA chains per thread, unrolled: the FP32 pipes, not the
// dependency latency, set the rate.  The result is stored only when it takes
// an impossible value, so the chains stay live without memory traffic.
__global__ void __launch_bounds__(256) fma_probe_kernel(float* out, int iters) {
    float a[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) a[c] = 1e-3f * (float)(threadIdx.x + c);
    const float m = 0.9999999f, k = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u)
#pragma unroll
            for (int c = 0; c < 8; ++c) a[c] = fmaf(a[c], m, k);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c) s += a[c];
    if (s == -1.f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int dstir_measure_fp32_rate(int32_t iters, double* flops_per_s, void* stream) {
    if (!flops_per_s || iters <= 0) return DSTIR_EINVAL;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return DSTIR_ECUDA;
    const int blocks = sms * 8, threads = 256;
    float* out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = DSTIR_OK;
    if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(float)) != cudaSuccess) return DSTIR_ENOMEM;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = DSTIR_ECUDA;
    if (rc == DSTIR_OK) {
        fma_probe_kernel<<<blocks, threads, 0, st>>>(out, iters);  // warm-up
        cudaEventRecord(e0, st);
        fma_probe_kernel<<<blocks, threads, 0, st>>>(out, iters);
        cudaEventRecord(e1, st);
        float ms = 0.f;
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess ||
            cudaGetLastError() != cudaSuccess || ms <= 0.f) {
            rc = DSTIR_ECUDA;
        } else {
            *flops_per_s = 2.0 * 8 * 16 * (double)iters * blocks * threads / (ms * 1e-3);
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    return rc;
}

extern "C" int dstir_measure_red_rate(int64_t n_nodes, int32_t reps, double* sectors_per_s, void* stream) {
    if (!sectors_per_s || n_nodes < 32 || reps <= 0) return DSTIR_EINVAL;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const long long rows = n_nodes / 32;
    float4* grid = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = DSTIR_OK;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return DSTIR_ECUDA;
    const int blocks = sms * 8, threads = 256;
    if (cudaMalloc(&grid, (size_t)rows * 32 * sizeof(float4)) != cudaSuccess) return DSTIR_ENOMEM;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = DSTIR_ECUDA;
    if (rc == DSTIR_OK) {
        cudaMemsetAsync(grid, 0, (size_t)rows * 32 * sizeof(float4), st);
        red_probe_kernel<<<blocks, threads, 0, st>>>(grid, rows, reps);  // warm-up
        cudaEventRecord(e0, st);
        red_probe_kernel<<<blocks, threads, 0, st>>>(grid, rows, reps);
        cudaEventRecord(e1, st);
        float ms = 0.f;
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess ||
            cudaGetLastError() != cudaSuccess || ms <= 0.f) {
            rc = DSTIR_ECUDA;
        } else {
            const double warps = (double)blocks * threads / 32.0;
            *sectors_per_s = warps * reps * 16.0 / (ms * 1e-3);
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(grid);
    return rc;
}
