// FP32 FMA throughput probe: the denominator of the soft-force kernel's
// roofline fraction.  Every thread runs 16 independent FFMA chains; the grid
// fills every SM with 8 blocks of 256 threads.  Flops = 2 per FMA.
#include <cuda_runtime.h>
#include <cstdint>

namespace {

constexpr int kChains = 16;

__global__ __launch_bounds__(256) void ffma_loop(float* out, int iters, float a, float b) {
    float v[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) v[c] = threadIdx.x * 1e-3f + c;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
#pragma unroll
            for (int c = 0; c < kChains; ++c) v[c] = fmaf(v[c], a, b);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += v[c];
    if (s == 123.456f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the loop live
}

// The same loop with packed FP32x2 FMAs (two FMAs per lane per instruction).
__global__ __launch_bounds__(256) void ffma2_loop(float* out, int iters, float a, float b) {
    float2 v[kChains / 2];
#pragma unroll
    for (int c = 0; c < kChains / 2; ++c) v[c] = make_float2(threadIdx.x * 1e-3f + c, threadIdx.x * 2e-3f + c);
    const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
#pragma unroll
            for (int c = 0; c < kChains / 2; ++c) v[c] = __ffma2_rn(v[c], a2, b2);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains / 2; ++c) s += v[c].x + v[c].y;
    if (s == 123.456f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" {

// Same measurement with packed FP32x2 FMAs (sm_100 and later).
int pgf_probe_fp32x2_peak(int iters, double* tflops, double* ms_out) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
    const int blocks = sms * 8, threads = 256;
    float* out = nullptr;
    if (cudaMalloc(&out, sizeof(float) * blocks * threads) != cudaSuccess) return 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    ffma2_loop<<<blocks, threads>>>(out, iters / 8 + 1, 0.999999f, 1e-7f);
    cudaEventRecord(e0);
    ffma2_loop<<<blocks, threads>>>(out, iters, 0.999999f, 1e-7f);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f) return 1;
    const double flops = 2.0 * kChains * 8.0 * (double)iters * blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    *ms_out = ms;
    return 0;
}

// Measures FP32 FMA throughput on the current device.  Returns 0 on success
// and writes TFLOP/s (2 flops per FMA) and the kernel time in ms.
int pgf_probe_fp32_peak(int iters, double* tflops, double* ms_out) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
    const int blocks = sms * 8, threads = 256;
    float* out = nullptr;
    if (cudaMalloc(&out, sizeof(float) * blocks * threads) != cudaSuccess) return 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    ffma_loop<<<blocks, threads>>>(out, iters / 8 + 1, 0.999999f, 1e-7f);  // warm-up
    cudaEventRecord(e0);
    ffma_loop<<<blocks, threads>>>(out, iters, 0.999999f, 1e-7f);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f) return 1;
    const double flops = 2.0 * kChains * 8.0 * (double)iters * blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    *ms_out = ms;
    return 0;
}

}  // extern "C"
