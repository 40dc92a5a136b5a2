// peak.cu -- measured FP32 and FP64 FMA-pipe peaks of the device: the
// denominators of the blind-rotation kernels' rooflines (split-FP32 form,
// plain FP64 form).
//
// The blind rotation is bound by the FP32 pipe and the shared-memory pipe,
// not by HBM or the tensor cores, so neither a copy bandwidth nor a GEMM
// rate is its roof.  This probe runs independent chains of packed FP32
// fused multiply-adds (fma.rn.f32x2: two lanes' FMAs in one instruction, the
// form the engine's transforms use) on every SM, 8 CTAs of 256 threads each,
// 16 chains a thread (enough independent work to cover the pipe latency at
// full occupancy), and times them with CUDA events.
#include <cuda_runtime.h>

#include "../../include/tfhe_gpu.h"

namespace {

constexpr int kChains = 16;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_fma_peak(float2 a, float2 b, int iters, float* sink) {
    float2 v[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i)
        v[i] = make_float2(threadIdx.x * 1e-7f + i, blockIdx.x * 1e-7f - i);
#pragma unroll 4
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < kChains; ++i) v[i] = __ffma2_rn(v[i], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += v[i].x + v[i].y;
    if (s == 1234.5f) sink[0] = s;  // keeps the chains alive; never true for these inputs
}

__global__ void __launch_bounds__(kThreads) k_fma_peak_fp64(double a, double b, int iters, double* sink) {
    double v[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) v[i] = threadIdx.x * 1e-9 + i - blockIdx.x * 1e-9;
#pragma unroll 4
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < kChains; ++i) v[i] = fma(v[i], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += v[i];
    if (s == 1234.5) sink[0] = s;  // keeps the chains alive; never true for these inputs
}

}  // namespace

// FP64 form of the probe: independent FP64 FMA chains (the plain FP64 form's
// transforms and products), same grid, 2 flops per FMA.
extern "C" tfhe_gpu_status tfhe_gpu_measure_fp64_peak(int32_t device, int32_t iters, double* tflops,
                                                      double* ms) {
    if (!tflops || iters < 1) return TFHE_GPU_BAD_PARAM;
    if (cudaSetDevice(device) != cudaSuccess) return TFHE_GPU_DEVICE_ERROR;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return TFHE_GPU_DEVICE_ERROR;
    double* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaStream_t st = nullptr;
    tfhe_gpu_status s = TFHE_GPU_OK;
    if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess) return TFHE_GPU_OOM;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        s = TFHE_GPU_DEVICE_ERROR;
    const int grid = sms * 8;
    float best = 0.f;
    for (int rep = 0; s == TFHE_GPU_OK && rep < 4; ++rep) {
        cudaEventRecord(e0, st);
        k_fma_peak_fp64<<<grid, kThreads, 0, st>>>(0.999999999, 1e-12, iters, sink);
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
            s = TFHE_GPU_DEVICE_ERROR;
            break;
        }
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (rep > 0 && (best == 0.f || t < best)) best = t;
    }
    if (s == TFHE_GPU_OK) {
        const double flops = 2.0 * kChains * (double)iters * grid * kThreads;
        *tflops = flops / (best * 1e-3) / 1e12;
        if (ms) *ms = best;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cudaFree(sink);
    return s;
}

extern "C" tfhe_gpu_status tfhe_gpu_measure_fp32_peak(int32_t device, int32_t iters, double* tflops,
                                                      double* ms) {
    if (!tflops || iters < 1) return TFHE_GPU_BAD_PARAM;
    if (cudaSetDevice(device) != cudaSuccess) return TFHE_GPU_DEVICE_ERROR;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return TFHE_GPU_DEVICE_ERROR;
    float* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaStream_t st = nullptr;
    tfhe_gpu_status s = TFHE_GPU_OK;
    if (cudaMalloc(&sink, sizeof(float)) != cudaSuccess) return TFHE_GPU_OOM;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        s = TFHE_GPU_DEVICE_ERROR;
    const int grid = sms * 8;
    const float2 a = make_float2(0.999999f, 1.000001f), b = make_float2(1e-7f, -1e-7f);
    float best = 0.f;
    for (int rep = 0; s == TFHE_GPU_OK && rep < 4; ++rep) {
        cudaEventRecord(e0, st);
        k_fma_peak<<<grid, kThreads, 0, st>>>(a, b, iters, sink);
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
            s = TFHE_GPU_DEVICE_ERROR;
            break;
        }
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (rep > 0 && (best == 0.f || t < best)) best = t;  // the first run warms up
    }
    if (s == TFHE_GPU_OK) {
        const double flops = 4.0 * kChains * (double)iters * grid * kThreads;  // 2 lanes x FMA
        *tflops = flops / (best * 1e-3) / 1e12;
        if (ms) *ms = best;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cudaFree(sink);
    return s;
}
