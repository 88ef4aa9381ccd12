// Complex arithmetic shared by the dense kernels (dense_z.cu) and the mixed-precision
// eigen-solver (eig_mixed.cu): element-type traits for double2 / float2, scalar overloads that
// keep FP32 instantiations in FP32, the complex helpers, the Givens generator and the QR
// deflation test.
#pragma once

#include <cuda_runtime.h>

#include "scw_dense.h"

namespace scw {
namespace z {

// element-type traits: scalar type, constructor, LAPACK's ulp (xLAMCH('P')) and safe minimum
template <typename C>
struct CT;
template <>
struct CT<double2> {
    using R = double;
    static __device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }
    static constexpr double ulp = 2.220446049250313e-16;
    static constexpr double safmin = 2.2250738585072014e-308;
};
template <>
struct CT<float2> {
    using R = float;
    static __device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
    static constexpr float ulp = 1.1920928955078125e-07f;
    static constexpr float safmin = 1.1754943508222875e-38f;
};

// scalar functions by overload, so that the FP32 instantiations stay in FP32
__device__ __forceinline__ double r_fma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float r_fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double r_abs(double a) { return fabs(a); }
__device__ __forceinline__ float r_abs(float a) { return fabsf(a); }
__device__ __forceinline__ double r_sqrt(double a) { return sqrt(a); }
__device__ __forceinline__ float r_sqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ double r_copysign(double a, double b) { return copysign(a, b); }
__device__ __forceinline__ float r_copysign(float a, float b) { return copysignf(a, b); }
__device__ __forceinline__ double r_max(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ float r_max(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double r_min(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float r_min(float a, float b) { return fminf(a, b); }

template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
    return CT<C>::mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C>
__device__ __forceinline__ C cmulc(C a, C b) {   // conj(a) * b
    return CT<C>::mk(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
template <typename C>
__device__ __forceinline__ C cadd(C a, C b) {
    return CT<C>::mk(a.x + b.x, a.y + b.y);
}
template <typename C>
__device__ __forceinline__ C csub(C a, C b) {
    return CT<C>::mk(a.x - b.x, a.y - b.y);
}
template <typename C>
__device__ __forceinline__ C cfma(C a, C b, C c) {   // a * b + c
    return CT<C>::mk(r_fma(a.x, b.x, r_fma(-a.y, b.y, c.x)), r_fma(a.x, b.y, r_fma(a.y, b.x, c.y)));
}
template <typename C>
__device__ __forceinline__ typename CT<C>::R cabs2(C a) {
    return a.x * a.x + a.y * a.y;
}
template <typename C>
__device__ __forceinline__ typename CT<C>::R cabs1(C a) {
    return r_abs(a.x) + r_abs(a.y);
}
template <typename C>
__device__ __forceinline__ C cdiv(C a, C b) {
    // Smith's algorithm
    if (r_abs(b.x) >= r_abs(b.y)) {
        const auto r = b.y / b.x, d = b.x + b.y * r;
        return CT<C>::mk((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    }
    const auto r = b.x / b.y, d = b.x * r + b.y;
    return CT<C>::mk((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
__device__ __forceinline__ bool skipped(const int* skip, int b) {
    return skip && skip[b];
}

template <typename C>
__device__ __forceinline__ void zlartg(C f, C g, typename CT<C>::R& c, C& s, C& r) {
    using R = typename CT<C>::R;
    // c s: [c, s; -conj(s), c] [f; g] = [r; 0], c real
    const R gf = cabs2(g);
    if (gf == 0) {
        c = 1;
        s = CT<C>::mk(0, 0);
        r = f;
        return;
    }
    const R ff = cabs2(f);
    if (ff == 0) {
        c = 0;
        const R ag = r_sqrt(gf);
        s = CT<C>::mk(g.x / ag, -g.y / ag);            // conj(g) / |g|
        r = CT<C>::mk(ag, 0);
        return;
    }
    const R af = r_sqrt(ff), d = r_sqrt(ff + gf);
    c = af / d;
    const C fs = CT<C>::mk(f.x / af, f.y / af);        // f / |f|
    s = cmulc(g, fs);                                   // conj(g) f / |f|  ... scaled below
    s = CT<C>::mk(s.x / d, s.y / d);
    r = CT<C>::mk(fs.x * d, fs.y * d);
}

// load of a matrix element: plain, or (kCg) through L2 only (ld.global.cg), for data that other
// CTAs of a thread-block cluster write between barriers
template <bool kCg>
__device__ __forceinline__ double2 hld(const double2* p) {
    if constexpr (kCg) return __ldcg(p);
    else return *p;
}
template <bool kCg>
__device__ __forceinline__ float2 hld(const float2* p) {
    if constexpr (kCg) return __ldcg(p);
    else return *p;
}

// deflation test for the subdiagonal entry h(k, k-1) of the active block ending at ihi
template <typename C, bool kCg = false>
__device__ __forceinline__ bool hqr_deflates(const C* H, int n, int k, int ihi) {
    using R = typename CT<C>::R;
    const R ulp = CT<C>::ulp;
    const R smlnum = CT<C>::safmin * ((R)n / ulp);
    const C hkk1 = hld<kCg>(H + (long long)k * n + k - 1);
    if (cabs1(hkk1) <= smlnum) return true;
    R tst = cabs1(hld<kCg>(H + (long long)(k - 1) * n + k - 1)) + cabs1(hld<kCg>(H + (long long)k * n + k));
    if (tst == 0) {
        if (k - 2 >= 0) tst += r_abs(hld<kCg>(H + (long long)(k - 1) * n + k - 2).x);
        if (k + 1 <= ihi) tst += r_abs(hld<kCg>(H + (long long)(k + 1) * n + k).x);
    }
    if (r_abs(hkk1.x) > ulp * tst) return false;
    // Ahues & Tisseur conservative deflation criterion (as in zlahqr)
    const C hk1k = hld<kCg>(H + (long long)(k - 1) * n + k);
    const C hkk = hld<kCg>(H + (long long)k * n + k);
    const C hk1k1 = hld<kCg>(H + (long long)(k - 1) * n + k - 1);
    const R ab = r_max(cabs1(hkk1), cabs1(hk1k));
    const R ba = r_min(cabs1(hkk1), cabs1(hk1k));
    const C dd = csub(hk1k1, hkk);
    const R aa = r_max(cabs1(hkk), cabs1(dd));
    const R bb = r_min(cabs1(hkk), cabs1(dd));
    const R s = aa + ab;
    if (ba * (ab / s) <= r_max(smlnum, ulp * (bb * (aa / s)))) return true;
    // coincident diagonal entries (bb = 0 above): zeroing the subdiagonal moves the two
    // eigenvalues by at most sqrt(|h(k,k-1) h(k-1,k)|), below rounding of h(k,k) when this
    // holds (a diagonal matrix with repeated eigenvalues and rounding-level couplings would
    // otherwise never deflate)
    return ba * ab <= (ulp * cabs1(hkk)) * (ulp * cabs1(hkk));
}

}  // namespace z
}  // namespace scw
