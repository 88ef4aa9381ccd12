// Measured issue peaks of the pipes the non-tensor kernels are bound by (no reference
// counterpart): the multi-function unit (MUFU) for sin / cos and, separately, for ex2 (the plain
// evaluator issues a sin and a cos per point and wave, and an ex2 only where the wave's k has an
// imaginary part in the plane), FP32 FMA and FP64 FMA.  Each kernel runs independent dependency
// chains per thread on every SM, long enough that launch overhead is negligible, and the rate
// is operations per second over the event-timed launch.
#include <cuda_runtime.h>

#include "scw_internal.h"

namespace scw {
namespace pk {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sin_approx(float x) {
    float y;
    asm volatile("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float cos_approx(float x) {
    float y;
    asm volatile("cos.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// per iteration and chain: one sin and one cos (kSinCos), or one ex2
template <bool kSinCos>
__global__ void __launch_bounds__(kThreads) mufu_kernel(float* out, int iters) {
    float v[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) v[c] = 0.001f * (threadIdx.x + 7 * c);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) v[c] = kSinCos ? cos_approx(sin_approx(v[c])) : ex2_approx(-v[c]);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += v[c];
    if (s == 12345.f) out[blockIdx.x] = s;     // keeps the chains live; never true in practice
}

__global__ void __launch_bounds__(kThreads) fma32_kernel(float* out, int iters) {
    float v[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) v[c] = 0.001f * (threadIdx.x + c);
    const float a = 0.999f, b = 1e-4f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) v[c] = fmaf(v[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += v[c];
    if (s == 12345.f) out[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kThreads) fma64_kernel(double* out, int iters) {
    double v[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) v[c] = 0.001 * (threadIdx.x + c);
    const double a = 0.999, b = 1e-4;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) v[c] = fma(v[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += v[c];
    if (s == 12345.0) out[blockIdx.x] = s;
}

}  // namespace pk
}  // namespace scw

using scw::fail;

extern "C" scw_status scw_measure_peaks(scw_ctx ctx, double* sincos_ops_per_s, double* ex2_ops_per_s,
                                        double* fp32_flops, double* fp64_flops) {
    using namespace scw::pk;
    if (!ctx) return fail(SCW_ERR_ARG, "scw_measure_peaks: null context");
    SCW_ON_DEVICE(ctx->device);
    const int blocks = ctx->sm_count * 8;
    void* out = nullptr;
    SCW_CUDA_TRY(cudaMalloc(&out, sizeof(double) * blocks));
    cudaEvent_t a = nullptr, b = nullptr;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
        if (a) cudaEventDestroy(a);
        cudaFree(out);
        return fail(SCW_ERR_CUDA, "scw_measure_peaks: event creation");
    }
    auto run = [&](int which, int iters, double ops_per_iter_thread, double* result) -> scw_status {
        for (int rep = 0; rep < 2; rep++) {      // the first launch warms up; the second is timed
            SCW_CUDA_TRY(cudaEventRecord(a, ctx->stream));
            if (which == 0) mufu_kernel<true><<<blocks, kThreads, 0, ctx->stream>>>((float*)out, iters);
            else if (which == 3) mufu_kernel<false><<<blocks, kThreads, 0, ctx->stream>>>((float*)out, iters);
            else if (which == 1) fma32_kernel<<<blocks, kThreads, 0, ctx->stream>>>((float*)out, iters);
            else fma64_kernel<<<blocks, kThreads, 0, ctx->stream>>>((double*)out, iters);
            SCW_CUDA_TRY(cudaGetLastError());
            ctx->launches++;
            SCW_CUDA_TRY(cudaEventRecord(b, ctx->stream));
        }
        SCW_CUDA_TRY(cudaEventSynchronize(b));
        float ms = 0.f;
        SCW_CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
        if (result) *result = (double)blocks * kThreads * iters * ops_per_iter_thread / (ms * 1e-3);
        return SCW_OK;
    };
    scw_status st = SCW_OK;
    if (st == SCW_OK && sincos_ops_per_s) st = run(0, 4096, 2.0 * kChains, sincos_ops_per_s);
    if (st == SCW_OK && ex2_ops_per_s) st = run(3, 8192, 1.0 * kChains, ex2_ops_per_s);
    if (st == SCW_OK && fp32_flops) st = run(1, 16384, 2.0 * kChains, fp32_flops);
    if (st == SCW_OK && fp64_flops) st = run(2, 1024, 2.0 * kChains, fp64_flops);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    return st;
}
