// FP64 complex dense linear algebra used by the per-layer solve (dense_z.cu).
#pragma once

#include <cuda_runtime.h>
#include <algorithm>

#include "scw_internal.h"

namespace scw {

// C = alpha A B + beta C (row-major, batched by strides in elements)
scw_status zgemm(cudaStream_t st, int M, int N, int K, double2 alpha, const double2* A, int lda, long long sA,
                 const double2* B, int ldb, long long sB, double2 beta, double2* C, int ldc, long long sC, int batch);
// in-place LU with partial pivoting of n x n matrices (leading dimension n); info[b] = first zero pivot + 1
scw_status zgetrf(cudaStream_t st, double2* A, int n, long long sA, int* piv, long long sP, int* info, int batch,
                  double2* work);
// B := A^-1 B using zgetrf's factors (B: n x nrhs, leading dimension nrhs)
scw_status zgetrs(cudaStream_t st, const double2* LU, int n, long long sA, const int* piv, long long sP, double2* B,
                  int nrhs, long long sB, int batch);
// eigenvalues W and right eigenvectors V (columns) of A (overwritten); work >= batch (n^2 + 3 n)
scw_status zgeev(cudaStream_t st, double2* A, double2* W, double2* V, int n, int batch, double2* work, int* status);

}  // namespace scw
