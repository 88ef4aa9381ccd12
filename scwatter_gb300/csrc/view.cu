// Display-side field processing of the viewer, on the GPU: scalar extraction
// (EvaluateScalarSlices, sCWatterView.cpp:300-352), range search (CalculateMinMax, :268-297)
// and colour mapping (EvaluateColorValue / EvaluateColorSlices, :200-265), writing device
// buffers instead of OpenGL textures.
#include <cfloat>
#include <cmath>
#include <algorithm>
#include <vector>

#include "scw_internal.h"

namespace scw {
namespace vw {

// S = E[.][c] for mode 0, 1, 2; |Ex|^2 + |Ey|^2 + |Ez|^2 (as a complex value, imaginary 0) for 3
__global__ void scalar_kernel(const float2* __restrict__ E, long long n, int mode, float2* __restrict__ S) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2* e = E + 3 * i;
    if (mode < 3) {
        S[i] = e[mode];
    } else {
        // E E* summed in complex<float> arithmetic: (a + ib)(a - ib) = a^2 + b^2 (+ 0i)
        // every product and sum rounded on its own (no fused multiply-add), as the host code does
        float s = 0.f;
        for (int c = 0; c < 3; c++) s = __fadd_rn(s, __fadd_rn(__fmul_rn(e[c].x, e[c].x), __fmul_rn(e[c].y, e[c].y)));
        S[i] = make_float2(s, 0.f);
    }
}

// per block (min re, max re, min im, max im); NaNs are skipped by the comparisons as in the
// reference's strict '<' / '>' tests
__global__ void minmax_kernel(const float2* __restrict__ S, long long n, float4* __restrict__ part) {
    __shared__ float4 sh[256];
    float4 m = make_float4(FLT_MAX, -FLT_MAX, FLT_MAX, -FLT_MAX);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = S[i];
        if (v.x < m.x) m.x = v.x;
        if (v.x > m.y) m.y = v.x;
        if (v.y < m.z) m.z = v.y;
        if (v.y > m.w) m.w = v.y;
    }
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            const float4 o = sh[threadIdx.x + s];
            float4 a = sh[threadIdx.x];
            a.x = fminf(a.x, o.x);
            a.y = fmaxf(a.y, o.y);
            a.z = fminf(a.z, o.z);
            a.w = fmaxf(a.w, o.w);
            sh[threadIdx.x] = a;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__device__ __forceinline__ float clamp01(float v) {
    if (isnan(v)) return 0.f;
    if (v < 0.f) return 0.f;
    if (v > 1.f) return 1.f;
    return v;
}

struct ColorParams {
    float real_low, real_high, imag_low, imag_high;
    float real_color[3], imag_color[3];
    int show_real, show_imag;
};

// RGB bytes: channel = 255 * (rn * real_color + in * imag_color), truncated as the float to
// unsigned char conversion of the reference does
__global__ void color_kernel(const float2* __restrict__ S, long long n, ColorParams p, unsigned char* __restrict__ rgb) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 v = S[i];
    const float rn = clamp01(__fdiv_rn(__fsub_rn(v.x, p.real_low), __fsub_rn(p.real_high, p.real_low)));
    const float in = clamp01(__fdiv_rn(__fsub_rn(v.y, p.imag_low), __fsub_rn(p.imag_high, p.imag_low)));
    for (int c = 0; c < 3; c++) {
        float x = 0.f;
        if (p.show_real) x = __fadd_rn(x, __fmul_rn(rn, p.real_color[c]));
        if (p.show_imag) x = __fadd_rn(x, __fmul_rn(in, p.imag_color[c]));
        rgb[3 * i + c] = (unsigned char)__fmul_rn(x, 255.f);
    }
}

}  // namespace vw
}  // namespace scw

using scw::fail;

extern "C" {

scw_status scw_view_scalar(scw_ctx ctx, const float* E, int64_t n, int mode, float* S) {
    if (!ctx || !E || !S || n < 0 || mode < 0 || mode > 3) return fail(SCW_ERR_ARG, "scw_view_scalar: bad arguments");
    if (n == 0) return SCW_OK;
    SCW_ON_DEVICE(ctx->device);
    scw::vw::scalar_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>((const float2*)E, n, mode, (float2*)S);
    SCW_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    return SCW_OK;
}

scw_status scw_view_minmax(scw_ctx ctx, const float* S, int64_t n, float* out4) {
    if (!ctx || !S || !out4 || n < 1) return fail(SCW_ERR_ARG, "scw_view_minmax: bad arguments");
    SCW_ON_DEVICE(ctx->device);
    const int blocks = (int)std::min<int64_t>(1024, (n + 255) / 256);
    scw_status st = ctx->scratch.reserve(sizeof(float4) * blocks);
    if (st != SCW_OK) return st;
    float4* part = (float4*)ctx->scratch.ptr;
    scw::vw::minmax_kernel<<<blocks, 256, 0, ctx->stream>>>((const float2*)S, n, part);
    SCW_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    std::vector<float4> h(blocks);
    SCW_CUDA_TRY(cudaMemcpyAsync(h.data(), part, sizeof(float4) * blocks, cudaMemcpyDeviceToHost, ctx->stream));
    SCW_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    float4 m = h[0];
    for (const auto& o : h) {
        m.x = std::fmin(m.x, o.x);
        m.y = std::fmax(m.y, o.y);
        m.z = std::fmin(m.z, o.z);
        m.w = std::fmax(m.w, o.w);
    }
    out4[0] = m.x;
    out4[1] = m.y;
    out4[2] = m.z;
    out4[3] = m.w;
    return SCW_OK;
}

// params: real_low, real_high, imag_low, imag_high, real_color[3], imag_color[3], show_real, show_imag
scw_status scw_view_color(scw_ctx ctx, const float* S, int64_t n, const float* params, unsigned char* rgb) {
    if (!ctx || !S || !params || !rgb || n < 0) return fail(SCW_ERR_ARG, "scw_view_color: bad arguments");
    if (n == 0) return SCW_OK;
    SCW_ON_DEVICE(ctx->device);
    scw::vw::ColorParams p{};
    p.real_low = params[0];
    p.real_high = params[1];
    p.imag_low = params[2];
    p.imag_high = params[3];
    for (int c = 0; c < 3; c++) {
        p.real_color[c] = params[4 + c];
        p.imag_color[c] = params[7 + c];
    }
    p.show_real = params[10] != 0.f;
    p.show_imag = params[11] != 0.f;
    scw::vw::color_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>((const float2*)S, n, p, rgb);
    SCW_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    return SCW_OK;
}

}  // extern "C"
