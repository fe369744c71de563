// i2_calibrate.cu -- measured pipe peaks and transcendental costs of the GPU in use, for the
// roofline of the pair kernels (the pair kernels are bounded by the FP64 / FP32 pipes, not by
// HBM or the tensor cores).  Each kernel runs independent dependency chains per thread so
// the pipe, not latency, limits it; timing uses CUDA events on a private stream.
#include "integrator2_gb300.h"

#include <cmath>
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;

__global__ void k_dfma(int iters, double *sink, double b, double c)
{
    double a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = threadIdx.x + k;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], b, c);
    double s = 0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == 1.2345) sink[0] = s;
}

__global__ void k_ffma(int iters, float *sink, float b, float c)
{
    float a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = threadIdx.x + k;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < kChains; ++k) a[k] = fmaf(a[k], b, c);
    float s = 0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == 1.2345f) sink[0] = s;
}

// f = 0 sqrt, 1 div, 2 log, 3 atan2, 4 sincos, 5 acos
template <int F>
__global__ void k_fn(int iters, double *sink)
{
    double a[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) a[k] = 0.3 + 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            double x = a[k];
            double y;
            if (F == 0) y = sqrt(x + 1.0);
            else if (F == 1) y = 1.0 / (x + 1.0);
            else if (F == 2) y = log(x + 1.0);
            else if (F == 3) y = atan2(x, 1.0 - 0.5 * x);
            else if (F == 4) { double s, c; sincos(x, &s, &c); y = s * c; }
            else y = acos(x - 0.5);
            a[k] = 0.5 * y + 0.25;  // stays in (0.25, 1)
        }
    double s = a[0] + a[1] + a[2] + a[3];
    if (s == 1.2345) sink[0] = s;
}

// f = 0 sqrtf, 1 divide, 2 log1pf, 3 atan2f, 4 logf
template <int F>
__global__ void k_fnf(int iters, float *sink)
{
    float a[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) a[k] = 0.3f + 1e-3f * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float x = a[k];
            float y;
            if (F == 0) y = sqrtf(x + 1.0f);
            else if (F == 1) y = 1.0f / (x + 1.0f);
            else if (F == 2) y = log1pf(x);
            else if (F == 3) y = atan2f(x, 1.0f - 0.5f * x);
            else y = logf(x + 1.0f);
            a[k] = 0.5f * y + 0.25f;
        }
    const float s = a[0] + a[1] + a[2] + a[3];
    if (s == 1.2345f) sink[0] = s;
}

template <class L>
float time_launch(L launch, cudaStream_t st)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    launch();  // warm-up
    cudaEventRecord(e0, st);
    launch();
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

} // namespace

extern "C" {

/* out[0] FP64 FMA TFLOP/s, out[1] FP32 FMA TFLOP/s, out[2..7] cost of one FP64 sqrt, divide,
 * log, atan2, sincos, acos in FP64-FMA time units, out[8..12] cost of one FP32 sqrtf, divide,
 * log1pf, atan2f, logf in FP32-FMA time units (out must hold 13 doubles) */
i2_status i2_calibrate_pipes(double *out)
{
    if (!out) return I2_ERR_INVALID_ARGUMENT;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return I2_ERR_CUDA;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return I2_ERR_CUDA;
    double *sink = nullptr;
    if (cudaMalloc(&sink, 64) != cudaSuccess) {
        cudaStreamDestroy(st);
        return I2_ERR_OUT_OF_MEMORY;
    }
    const int blocks = sms * 8, tpb = 256;
    const double threads = (double)blocks * tpb;
    const int it64 = 2048, it32 = 65536, itf = 512;
    const float t64 = time_launch([&] { k_dfma<<<blocks, tpb, 0, st>>>(it64, sink, 0.999999, 1e-7); }, st);
    const float t32 = time_launch([&] { k_ffma<<<blocks, tpb, 0, st>>>(it32, (float *)sink, 0.999999f, 1e-7f); }, st);
    const double fma_ms = t64 / (threads * it64 * kChains);  // ms per FP64 FMA (throughput)
    out[0] = 2.0 * threads * it64 * kChains / (t64 * 1e-3) / 1e12;
    out[1] = 2.0 * threads * it32 * kChains / (t32 * 1e-3) / 1e12;
    float tf[6];
    tf[0] = time_launch([&] { k_fn<0><<<blocks, tpb, 0, st>>>(itf, sink); }, st);
    tf[1] = time_launch([&] { k_fn<1><<<blocks, tpb, 0, st>>>(itf, sink); }, st);
    tf[2] = time_launch([&] { k_fn<2><<<blocks, tpb, 0, st>>>(itf, sink); }, st);
    tf[3] = time_launch([&] { k_fn<3><<<blocks, tpb, 0, st>>>(itf, sink); }, st);
    tf[4] = time_launch([&] { k_fn<4><<<blocks, tpb, 0, st>>>(itf, sink); }, st);
    tf[5] = time_launch([&] { k_fn<5><<<blocks, tpb, 0, st>>>(itf, sink); }, st);
    for (int f = 0; f < 6; ++f) out[2 + f] = tf[f] / (threads * itf * 4) / fma_ms;
    // FP32: time of one sqrtf, divide, log1pf, atan2f, logf in units of one FP32 FMA
    const int itf32 = 4096;
    const double ffma_ms = t32 / (threads * (double)it32 * kChains);
    float tg[5];
    tg[0] = time_launch([&] { k_fnf<0><<<blocks, tpb, 0, st>>>(itf32, (float *)sink); }, st);
    tg[1] = time_launch([&] { k_fnf<1><<<blocks, tpb, 0, st>>>(itf32, (float *)sink); }, st);
    tg[2] = time_launch([&] { k_fnf<2><<<blocks, tpb, 0, st>>>(itf32, (float *)sink); }, st);
    tg[3] = time_launch([&] { k_fnf<3><<<blocks, tpb, 0, st>>>(itf32, (float *)sink); }, st);
    tg[4] = time_launch([&] { k_fnf<4><<<blocks, tpb, 0, st>>>(itf32, (float *)sink); }, st);
    for (int f = 0; f < 5; ++f) out[8 + f] = tg[f] / (threads * (double)itf32 * 4) / ffma_ms;
    const cudaError_t e = cudaGetLastError();
    cudaFree(sink);
    cudaStreamDestroy(st);
    return e == cudaSuccess ? I2_OK : I2_ERR_CUDA;
}

} // extern "C"
