// oxg_peaks.cu - throughput microbenchmarks of the two pipes the MD step is bound by:
// FP32 FMA and the special-function unit. They give the denominators of the step's
// compute roofline on the device it runs on (the measured HBM and tensor peaks say
// nothing about either).
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/oxdna_gb300.h"
#include "oxg_internal.h"

namespace {

constexpr int kChains = 8;   // independent dependency chains per thread
constexpr int kUnroll = 16;  // operations per chain per loop trip

// kChains x kUnroll dependent FMAs per trip; b slightly below 1 keeps the values bounded.
__global__ void __launch_bounds__(256) k_peak_fma(float* sink, int trips, float b, float c)
{
    float a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = 1e-3f * (float)(threadIdx.x + k);
    for (int t = 0; t < trips; ++t) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
#pragma unroll
            for (int k = 0; k < kChains; ++k) a[k] = fmaf(a[k], b, c);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == -1.f) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

// kChains x kUnroll dependent reciprocal square roots (one special-function op each;
// the iteration x <- x^-1/2 converges to 1).
__global__ void __launch_bounds__(256) k_peak_sfu(float* sink, int trips)
{
    float a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = 1.5f + 1e-3f * (float)(threadIdx.x + k);
    for (int t = 0; t < trips; ++t) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
#pragma unroll
            for (int k = 0; k < kChains; ++k) asm("rsqrt.approx.ftz.f32 %0, %0;" : "+f"(a[k]));
        }
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == -1.f) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int oxg_device_peaks(double* out, int n, void* stream)
{
    if (!out || n < 1) return oxg::internal_set_error(OXG_ERR_INVALID_ARG, "bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    const int threads = 256, blocks = oxg::internal_num_sms() * 8;  // 16 warps per SMSP
    float* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = OXG_OK;
    double res[2] = {0.0, 0.0};
    if (cudaMalloc(&sink, sizeof(float) * blocks * threads) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        rc = oxg::internal_set_error(OXG_ERR_CUDA, "peak benchmark setup failed");
    }
    for (int which = 0; which < 2 && rc == OXG_OK && which < n; ++which) {
        const int trips = which == 0 ? 2048 : 512;
        float best = 1e30f;
        for (int rep = 0; rep < 4 && rc == OXG_OK; ++rep) {  // rep 0 warms up
            cudaEventRecord(e0, s);
            if (which == 0) k_peak_fma<<<blocks, threads, 0, s>>>(sink, trips, 0.99999f, 1e-6f);
            else k_peak_sfu<<<blocks, threads, 0, s>>>(sink, trips);
            cudaEventRecord(e1, s);
            float ms = 0.f;
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
                rc = oxg::internal_set_error(OXG_ERR_CUDA, "peak benchmark launch failed");
                break;
            }
            if (rep > 0) best = std::min(best, ms);
        }
        const double ops = (double)blocks * threads * trips * kUnroll * kChains;
        // FMA: 2 flops each (GFLOP/s); special function: 1 op each (Gop/s)
        res[which] = (which == 0 ? 2.0 : 1.0) * ops / (best * 1e-3) / 1e9;
    }
    for (int k = 0; k < 2 && k < n; ++k) out[k] = res[k];
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (sink) cudaFree(sink);
    return rc;
}
