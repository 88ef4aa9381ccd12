// FP64 complex dense linear algebra used by the per-layer solve (dense_z.cu).
#pragma once

#include <cuda_runtime.h>
#include <algorithm>

#include "scw_internal.h"

namespace scw {

#ifdef __CUDACC__
// principal square root without cancellation: the larger of |Re|, |Im| of the root comes from
// sqrt((|Re a| + |a|) / 2), the other from Im a / (2 x)
__device__ __forceinline__ double2 zsqrt(double2 a) {
    if (a.x == 0.0 && a.y == 0.0) return make_double2(0.0, 0.0);
    const double t = sqrt(0.5 * (fabs(a.x) + hypot(a.x, a.y)));
    if (a.x >= 0.0) return make_double2(t, a.y / (2.0 * t));
    return make_double2(fabs(a.y) / (2.0 * t), copysign(t, a.y));
}
__device__ __forceinline__ float2 zsqrt(float2 a) {
    if (a.x == 0.0f && a.y == 0.0f) return make_float2(0.0f, 0.0f);
    const float t = sqrtf(0.5f * (fabsf(a.x) + hypotf(a.x, a.y)));
    if (a.x >= 0.0f) return make_float2(t, a.y / (2.0f * t));
    return make_float2(fabsf(a.y) / (2.0f * t), copysignf(t, a.y));
}
#endif

// The kernels are templates over the complex element type: double2 (FP64, the solve's
// precision) or float2 (FP32, the first stage of the mixed-precision eigen-solver).  A
// non-null skip[b] != 0 makes every kernel leave batch entry b untouched.

// C = alpha A B + beta C (row-major, batched by strides in elements)
template <typename C>
scw_status gemm(cudaStream_t st, int M, int N, int K, C alpha, const C* A, int lda, long long sA, const C* B, int ldb,
                long long sB, C beta, C* Cm, int ldc, long long sC, int batch, const int* skip = nullptr);
// in-place LU with partial pivoting of n x n matrices (leading dimension n); info[b] = first zero pivot + 1
template <typename C>
scw_status getrf(cudaStream_t st, C* A, int n, long long sA, int* piv, long long sP, int* info, int batch);
// B := A^-1 B using getrf's factors (B: n x nrhs, leading dimension nrhs)
template <typename C>
scw_status getrs(cudaStream_t st, const C* LU, int n, long long sA, const int* piv, long long sP, C* B, int nrhs,
                 long long sB, int batch);
// eigenvalues W and right eigenvectors V (columns) of A (overwritten); work >= batch (n^2 + 3 n);
// status[b] = 1 when the QR iteration did not converge.  wide: the Hessenberg reduction of
// matrices with n >= kWideMinN is spread over the whole GPU (3 launches per column) instead of one
// CTA per matrix -- for batches too small to fill the SMs; a batch graph with many concurrent
// items keeps the one-CTA form (fewer nodes).
constexpr int kWideMinN = 128;
template <typename C>
scw_status geev(cudaStream_t st, C* A, C* W, C* V, int n, int batch, C* work, int* status, const int* skip = nullptr,
                bool wide = false);

inline scw_status zgemm(cudaStream_t st, int M, int N, int K, double2 alpha, const double2* A, int lda, long long sA,
                        const double2* B, int ldb, long long sB, double2 beta, double2* C, int ldc, long long sC,
                        int batch) {
    return gemm<double2>(st, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch);
}
inline scw_status zgetrf(cudaStream_t st, double2* A, int n, long long sA, int* piv, long long sP, int* info,
                         int batch, double2* /*unused*/) {
    return getrf<double2>(st, A, n, sA, piv, sP, info, batch);
}
inline scw_status zgetrs(cudaStream_t st, const double2* LU, int n, long long sA, const int* piv, long long sP,
                         double2* B, int nrhs, long long sB, int batch) {
    return getrs<double2>(st, LU, n, sA, piv, sP, B, nrhs, sB, batch);
}
inline scw_status zgeev(cudaStream_t st, double2* A, double2* W, double2* V, int n, int batch, double2* work,
                        int* status, bool wide = false) {
    return geev<double2>(st, A, W, V, n, batch, work, status, nullptr, wide);
}
// Hessenberg form of A (in place, n x n per batch entry) and the unitary Q (A = Q H Q^H);
// work >= batch * 3 n
scw_status zgehrd(cudaStream_t st, double2* A, double2* Q, int n, int batch, double2* work);

}  // namespace scw
