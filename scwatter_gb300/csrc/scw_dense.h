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
#endif

// C = alpha A B + beta C (row-major, batched by strides in elements)
scw_status zgemm(cudaStream_t st, int M, int N, int K, double2 alpha, const double2* A, int lda, long long sA,
                 const double2* B, int ldb, long long sB, double2 beta, double2* C, int ldc, long long sC, int batch);
// in-place LU with partial pivoting of n x n matrices (leading dimension n); info[b] = first zero pivot + 1
scw_status zgetrf(cudaStream_t st, double2* A, int n, long long sA, int* piv, long long sP, int* info, int batch,
                  double2* work);
// B := A^-1 B using zgetrf's factors (B: n x nrhs, leading dimension nrhs)
scw_status zgetrs(cudaStream_t st, const double2* LU, int n, long long sA, const int* piv, long long sP, double2* B,
                  int nrhs, long long sB, int batch);
// Hessenberg form of A (in place, n x n per batch entry) and the unitary Q (A = Q H Q^H);
// work >= batch * 3 n
scw_status zgehrd(cudaStream_t st, double2* A, double2* Q, int n, int batch, double2* work);
// eigenvalues W and right eigenvectors V (columns) of A (overwritten); work >= batch (n^2 + 3 n)
scw_status zgeev(cudaStream_t st, double2* A, double2* W, double2* V, int n, int batch, double2* work, int* status);

}  // namespace scw
