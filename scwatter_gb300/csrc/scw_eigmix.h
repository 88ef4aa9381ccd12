// Mixed-precision eigen-solver of batched dense complex matrices (eig_mixed.cu).
//
// GB300 issues FP64 at about 1/64 of its FP32 rate, and the Householder + QR eigen-solve of a
// layer matrix is inherently one CTA per matrix.  So the O(n^3) factorisation runs in FP32,
// and FP64 accuracy comes back through Newton refinement of all eigenpairs at once, which
// costs one FP64 GEMM per step spread over every SM:
//   R = A X - X diag(lambda)          (FP64 GEMM)
//   E = X^-1 R                        (FP32 LU of X)
//   lambda_i += E_ii, X += X F,  F_ij = E_ij / (lambda_j - lambda_i)   (FP32 GEMM, FP64 sum)
// Eigenvalues closer than tau_rel * ||A||_1 form clusters.  Within a cluster the k x k block
// diag(lambda) + E is solved in FP64 by a small Schur decomposition.  Its eigenvectors then
// rotate the cluster's columns.  A slice stops refining when every column's relative residual
// ||A x - lambda x|| / (||A||_1 ||x||) is at most tol, and after the last step it is accepted
// when that residual is at most tol_accept.  Otherwise (FP32 QR not converged, a cluster above
// kMaxCluster, a singular X, no convergence within the step limit) that slice goes through the
// FP64 Householder + QR solver.
#pragma once

#include <cuda_runtime.h>

#include "scw_internal.h"

namespace scw {
namespace mx {

constexpr int kMaxCluster = 64;     // largest cluster solved in place
constexpr int kMaxN = 4096;         // largest matrix taken by the mixed path

struct EigMixWs {
    // four FP32 n x n slots per matrix (S0 and S1 adjacent: together one FP64 n x n slot)
    float2 *S0, *S1, *S2, *S3;
    float2 *hw;                     // 3 n per matrix, directly after S1 (FP32 QR work)
    float2 *lam32;                  // n per matrix
    int *label, *member, *cstart, *ncl, *piv, *info, *qr, *state, *steps;
    double2* Y;                     // kMaxCluster * n per matrix: cluster eigenvector blocks
    double *rn, *xn, *anorm, *res;  // column residual / norm sums, ||A||_1, max residual
};

// bytes of the small buffers (everything but S0..S3, hw, lam32) for Z matrices of order n
size_t eigmix_small_bytes(int n, int Z);
// carves the small buffers from base (which must be 256-byte aligned); big slots are set by the caller
void eigmix_carve_small(EigMixWs& w, char* base, int n, int Z);

struct EigMixParams {
    int steps = 10;                 // refinement steps (each begins with the residual check); converged
                                    // slices skip the rest, and a step costs about 1/50 of the FP64 QR
                                    // fallback that a slow slice would otherwise take
    int steps_large = 16;           // the same for n >= kLargeN: dense spectra there converge linearly
                                    // (about 3x per step from an FP32 start), so more steps pay
    static constexpr int kLargeN = 1600;
    double tau_rel = 1e-5;          // cluster threshold relative to ||A||_1
    double deg_rel = 1e-12;         // within a cluster: eigenvalues this close count as equal
    double tol = 1e-14;             // a slice stops refining once its max relative column residual is this small
    double tol_accept = 1e-12;      // from step `steps` on: accepted at or below this; after the last
                                    // step, else the FP64 solver
    bool wide = false;              // Hessenberg reductions spread over the GPU (see geev)
};

// Eigenpairs of Z matrices A (n x n, row-major, preserved unless a matrix falls back) into
// lam (n per matrix) and V (n x n, columns).  fb_work: the FP64 fallback's work, >= Z (n^2 + 3 n)
// double2, and it may alias S0..S3 / hw.  status[b] = 1 if even the FP64 fallback failed.
// Launches only (graph-capturable); *launches is incremented by the kernels issued.
scw_status geev_mixed(cudaStream_t st, double2* A, double2* lam, double2* V, int n, int Z, const EigMixWs& w,
                      double2* fb_work, int* status, const EigMixParams& prm, long long* launches);

}  // namespace mx
}  // namespace scw
