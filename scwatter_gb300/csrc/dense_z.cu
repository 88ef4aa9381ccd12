// FP64 complex dense linear algebra on the GPU, written for the per-layer coupled-wave solve:
// batched GEMM, blocked LU with partial pivoting and solves, and the non-Hermitian eigenvalue
// problem (Householder Hessenberg reduction, single-shift complex QR with Schur vectors,
// triangular eigenvectors, back-transformation).  They replace the MKL LAPACKE_zgeev,
// LAPACKE_zgesv and cblas_zgemm calls of the reference (third_Lapack.h:38-87).
//
// Conventions: row-major storage, element (i, j) of a matrix with leading dimension ld at
// A[i * ld + j]; complex numbers are double2 (re, im); "batched" kernels take a batch stride in
// elements and run one matrix per blockIdx.z (GEMM) or per CTA (factorisations).
//
// The GB300 FP64 rate is low (about 8 GFLOP/s per SM), so the O(n^3) parts are spread over all
// SMs where the algorithm allows it (GEMM, the trailing updates of LU); the inherently
// sequential ones (Hessenberg reduction, QR sweeps) run one CTA per matrix and are batched over
// the slices of a sample.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <vector>

#include <cooperative_groups.h>

#include "scw_dense.h"
#include "scw_complex.cuh"

namespace scw {
namespace z {

// ------------------------------------------------------------------------------------
// GEMM: C = alpha * op(A) * B + beta * C, op = identity.  64 x 64 tiles, 256 threads, each
// thread a 4 x 4 complex block; K staged 16 at a time through shared memory.
// ------------------------------------------------------------------------------------
constexpr int kGT = 64, kGK = 16;

template <typename C>
__global__ void __launch_bounds__(256)
gemm_kernel(int M, int N, int K, C alpha, const C* __restrict__ A, int lda, long long sA, const C* __restrict__ B,
            int ldb, long long sB, C beta, C* __restrict__ Cm, int ldc, long long sC, const int* __restrict__ skip) {
    if (skipped(skip, blockIdx.z)) return;
    __shared__ C As[kGK][kGT + 1];
    __shared__ C Bs[kGK][kGT + 1];
    A += sA * blockIdx.z;
    B += sB * blockIdx.z;
    Cm += sC * blockIdx.z;
    const int i0 = blockIdx.y * kGT, j0 = blockIdx.x * kGT;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const C zero = CT<C>::mk(0, 0);
    C acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = zero;
    for (int k0 = 0; k0 < K; k0 += kGK) {
        for (int e = threadIdx.x; e < kGK * kGT; e += 256) {
            const int r = e / kGK, kk = e % kGK;         // A tile: rows i0 + r, cols k0 + kk
            const int gi = i0 + r, gk = k0 + kk;
            As[kk][r] = (gi < M && gk < K) ? A[(long long)gi * lda + gk] : zero;
            const int kk2 = e / kGT, c = e % kGT;         // B tile: rows k0 + kk2, cols j0 + c
            const int gk2 = k0 + kk2, gj = j0 + c;
            Bs[kk2][c] = (gk2 < K && gj < N) ? B[(long long)gk2 * ldb + gj] : zero;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kGK; kk++) {
            C a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                a[q] = As[kk][ty + 16 * q];
                b[q] = Bs[kk][tx + 16 * q];
            }
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++) acc[p][q] = cfma(a[p], b[q], acc[p][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; p++) {
        const int gi = i0 + ty + 16 * p;
        if (gi >= M) continue;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int gj = j0 + tx + 16 * q;
            if (gj >= N) continue;
            C* c = Cm + (long long)gi * ldc + gj;
            C v = cmul(alpha, acc[p][q]);
            if (beta.x != 0 || beta.y != 0) v = cfma(beta, *c, v);
            *c = v;
        }
    }
}

// ------------------------------------------------------------------------------------
// LU with partial pivoting, blocked (panel width kNB), batched: one CTA per matrix for the
// panel factorisation and the row-swap / triangular-solve kernels, batched GEMM for the
// trailing update.  piv[k] = row swapped with row k at step k (LAPACK convention, 0-based).
// info[b] = first zero pivot + 1 (0: nonsingular).
// ------------------------------------------------------------------------------------
constexpr int kNB = 32;

template <typename C>
__global__ void __launch_bounds__(512)
lu_panel_kernel(C* __restrict__ A, int n, int lda, long long sA, int k0, int nb, int* __restrict__ piv, long long sP,
                int* __restrict__ info) {
    using R = typename CT<C>::R;
    A += sA * blockIdx.x;
    piv += sP * blockIdx.x;
    __shared__ R red_v[16];
    __shared__ int red_i[16];
    __shared__ C pivrow[kNB];
    for (int k = k0; k < k0 + nb; k++) {
        // pivot search over rows k..n-1 of column k
        R best = -1;
        int bi = k;
        for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
            const R v = cabs1(A[(long long)i * lda + k]);
            if (v > best) {
                best = v;
                bi = i;
            }
        }
        // arg-max (largest |a|, then smallest row): butterfly within each warp, then over the
        // warps' winners
        for (int o = 16; o > 0; o >>= 1) {
            const R ov = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) {
                best = ov;
                bi = oi;
            }
        }
        if ((threadIdx.x & 31) == 0) {
            red_v[threadIdx.x >> 5] = best;
            red_i[threadIdx.x >> 5] = bi;
        }
        __syncthreads();
        R pv = red_v[0];
        int p = red_i[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++)
            if (red_v[w] > pv || (red_v[w] == pv && red_i[w] < p)) {
                pv = red_v[w];
                p = red_i[w];
            }
        const bool zero = pv == 0;
        if (threadIdx.x == 0) {
            piv[k] = p;
            if (zero && info[blockIdx.x] == 0) info[blockIdx.x] = k + 1;
        }
        // swap rows k and p inside the panel columns k0 .. k0+nb-1
        if (p != k) {
            for (int j = k0 + threadIdx.x; j < k0 + nb; j += blockDim.x) {
                const C t = A[(long long)k * lda + j];
                A[(long long)k * lda + j] = A[(long long)p * lda + j];
                A[(long long)p * lda + j] = t;
            }
        }
        __syncthreads();
        const C d = A[(long long)k * lda + k];
        for (int j = k + 1 + threadIdx.x; j < k0 + nb; j += blockDim.x) pivrow[j - k0] = A[(long long)k * lda + j];
        __syncthreads();
        // scale the column below the pivot and update the remaining panel columns
        const C inv = zero ? CT<C>::mk(0, 0) : cdiv(CT<C>::mk(1, 0), d);
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) {
            C* row = A + (long long)i * lda;
            const C l = cmul(row[k], inv);
            row[k] = l;
            for (int j = k + 1; j < k0 + nb; j++) row[j] = csub(row[j], cmul(l, pivrow[j - k0]));
        }
        __syncthreads();
    }
}

// apply the panel's swaps to the columns outside the panel, then solve L11 U12 = A12
template <typename C>
__global__ void __launch_bounds__(256)
lu_swap_trsm_kernel(C* __restrict__ A, int n, int lda, long long sA, int k0, int nb, const int* __restrict__ piv,
                    long long sP) {
    A += sA * blockIdx.y;
    piv += sP * blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;    // one column per thread
    if (j >= n || (j >= k0 && j < k0 + nb)) return;
    for (int k = k0; k < k0 + nb; k++) {
        const int p = piv[k];
        if (p != k) {
            const C t = A[(long long)k * lda + j];
            A[(long long)k * lda + j] = A[(long long)p * lda + j];
            A[(long long)p * lda + j] = t;
        }
    }
    if (j < k0 + nb) return;                                // columns left of the panel: swaps only
    for (int k = k0; k < k0 + nb; k++) {                    // unit lower triangular solve
        C v = A[(long long)k * lda + j];
        for (int m = k0; m < k; m++) v = csub(v, cmul(A[(long long)k * lda + m], A[(long long)m * lda + j]));
        A[(long long)k * lda + j] = v;
    }
}

// Row interchanges of B from getrf's pivots (LAPACK laswp order), one thread per column.
template <typename C>
__global__ void __launch_bounds__(256)
laswp_kernel(const int* __restrict__ piv, long long sP, C* __restrict__ B, int ldb, long long sB, int n, int nrhs) {
    piv += sP * blockIdx.y;
    B += sB * blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nrhs) return;
    for (int k = 0; k < n; k++) {
        const int p = piv[k];
        if (p != k) {
            const C t = B[(long long)k * ldb + j];
            B[(long long)k * ldb + j] = B[(long long)p * ldb + j];
            B[(long long)p * ldb + j] = t;
        }
    }
}

// Triangular solve restricted to the diagonal block rows [k0, k0 + nb) of the LU factors, one
// thread per right-hand-side column: unit lower L (upper == 0) or U (upper == 1).  Rows
// outside the block were already folded in by the GEMM updates of the blocked solve.
template <typename C>
__global__ void __launch_bounds__(256)
trsm_block_kernel(const C* __restrict__ LU, int lda, long long sA, int k0, int nb, C* __restrict__ B, int ldb,
                  long long sB, int nrhs, int upper) {
    LU += sA * blockIdx.y;
    B += sB * blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nrhs) return;
    if (!upper) {
        for (int i = k0; i < k0 + nb; i++) {
            C v = B[(long long)i * ldb + j];
            const C* row = LU + (long long)i * lda;
            for (int m = k0; m < i; m++) v = csub(v, cmul(row[m], B[(long long)m * ldb + j]));
            B[(long long)i * ldb + j] = v;
        }
    } else {
        for (int i = k0 + nb - 1; i >= k0; i--) {
            C v = B[(long long)i * ldb + j];
            const C* row = LU + (long long)i * lda;
            for (int m = i + 1; m < k0 + nb; m++) v = csub(v, cmul(row[m], B[(long long)m * ldb + j]));
            B[(long long)i * ldb + j] = cdiv(v, row[i]);
        }
    }
}

// ------------------------------------------------------------------------------------
// Hessenberg reduction A -> Q^H A Q (zgehd2 semantics: H(k) = I - tau v v^H, v(k+1) = 1),
// one CTA per matrix, with the explicit unitary Q accumulated (Q := Q H(k)).
// ------------------------------------------------------------------------------------
template <typename R>
__device__ R block_sum(R v, R* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    R s = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sh[i];
    return s;
}

// y[i] = tau * sum_{j >= j0} M[i][j] v[j] for every row i: a warp per row, lanes along the row
// (coalesced), then a butterfly sum
template <typename C>
__device__ __forceinline__ void row_products(const C* __restrict__ M, const C* __restrict__ v, C* __restrict__ y, int n,
                                             int j0, C tau) {
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int i = threadIdx.x >> 5; i < n; i += nw) {
        const C* row = M + (long long)i * n;
        C s = CT<C>::mk(0, 0);
#pragma unroll 4
        for (int j = j0 + lane; j < n; j += 32) s = cfma(row[j], v[j], s);
        for (int o = 16; o > 0; o >>= 1) {
            s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
            s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
        }
        if (lane == 0) y[i] = cmul(tau, s);
    }
}

// col[i * ld] += u[i] * alpha for i in [i0, i1): kStripe rows at a time, loads before the
// updates, so that a thread has kStripe independent loads in flight instead of one
// load-update-store chain per row
template <typename C>
__device__ __forceinline__ void column_axpy(C* __restrict__ col, long long ld, int i0, int i1, const C* __restrict__ u,
                                            C alpha) {
    constexpr int kStripe = sizeof(typename CT<C>::R) == sizeof(float) ? 8 : 4;
    for (int b = i0; b < i1; b += kStripe) {
        C a[kStripe];
#pragma unroll
        for (int q = 0; q < kStripe; q++)
            if (b + q < i1) a[q] = col[(long long)(b + q) * ld];
#pragma unroll
        for (int q = 0; q < kStripe; q++)
            if (b + q < i1) col[(long long)(b + q) * ld] = cfma(u[b + q], alpha, a[q]);
    }
}

template <typename C>
__global__ void __launch_bounds__(1024)
hessenberg_kernel(C* __restrict__ A, C* __restrict__ Q, int n, long long sA, C* __restrict__ work,
                  const int* __restrict__ skip) {
    using R = typename CT<C>::R;
    if (skipped(skip, blockIdx.x)) return;
    A += sA * blockIdx.x;
    Q += sA * blockIdx.x;
    C* v = work + (long long)blockIdx.x * 3 * n;      // Householder vector (rows k+1..n-1)
    C* y = v + 2 * n;                                   // tau A v / tau Q v (the work keeps 3 n per matrix)
    __shared__ R sh[32];
    __shared__ C s_tau, s_beta;
    // FP32 (first stage of the mixed solver): a column whose part below the diagonal is under
    // ulp ||A||_F / sqrt(n) (ulp times the root-mean-square row norm) is set to zero instead of
    // reflected.  That is a backward error of rounding size, and it keeps a (nearly) diagonal
    // matrix, e.g. the reduced matrix of a homogeneous layer whose off-diagonal entries are DFT
    // rounding, from being scrambled by reflectors built from noise.  (ulp ||A||_F itself grows as
    // sqrt(n) and at n = 3200 dropped real couplings.)  FP64 keeps zgehd2's behaviour.
    constexpr bool kDropNegligible = sizeof(R) == sizeof(float);
    constexpr int kStripe = sizeof(R) == sizeof(float) ? 8 : 4;
    R neg2 = 0;
    if (kDropNegligible) {
        R a2 = 0;
        for (long long i = threadIdx.x; i < (long long)n * n; i += blockDim.x) a2 += cabs2(A[i]);
        neg2 = block_sum(a2, sh) * CT<C>::ulp * CT<C>::ulp / (R)n;
    }
    for (int i = threadIdx.x; i < n * n; i += blockDim.x) Q[i] = CT<C>::mk((i / n) == (i % n) ? 1 : 0, 0);
    __syncthreads();
    for (int k = 0; k + 2 < n; k++) {
        // Householder for x = A[k+1:n, k] (zlarfg)
        R xn2 = 0;
        for (int i = k + 2 + threadIdx.x; i < n; i += blockDim.x) xn2 += cabs2(A[(long long)i * n + k]);
        xn2 = block_sum(xn2, sh);
        const C alpha = A[(long long)(k + 1) * n + k];
        if (kDropNegligible && xn2 + cabs2(alpha) <= neg2) {
            for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[(long long)i * n + k] = CT<C>::mk(0, 0);
            __syncthreads();
            continue;
        }
        if (threadIdx.x == 0) {
            if (xn2 == 0 && alpha.y == 0) {
                s_tau = CT<C>::mk(0, 0);
                s_beta = alpha;
            } else {
                const R beta = -r_copysign(r_sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
                s_tau = CT<C>::mk((beta - alpha.x) / beta, -alpha.y / beta);
                s_beta = CT<C>::mk(beta, 0);
            }
        }
        __syncthreads();
        const C tau = s_tau;
        if (tau.x == 0 && tau.y == 0) {
            __syncthreads();
            continue;
        }
        const C scal = cdiv(CT<C>::mk(1, 0), csub(alpha, s_beta));
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x)
            v[i] = (i == k + 1) ? CT<C>::mk(1, 0) : cmul(A[(long long)i * n + k], scal);
        __syncthreads();
        // right: A[:, k+1:] -= tau (A[:, k+1:] v) v^H   (all rows; a warp per row for the products)
        row_products(A, v, y, n, k + 1, tau);
        __syncthreads();
        // then left: A[k+1:, k+1:] -= conj(tau) v (v^H A[k+1:, k+1:]).  Both act on one column
        // at a time, so each thread owns its columns: right update (all rows) while summing
        // v^H of the updated column, then the left update of that column.
        for (int j = k + 1 + threadIdx.x; j < n; j += blockDim.x) {
            const C vc = CT<C>::mk(v[j].x, -v[j].y);
            C s = CT<C>::mk(0, 0);
            C* col = A + j;
            // kStripe rows at a time: loads first, then the updates (see column_axpy)
            for (int i0 = 0; i0 < n; i0 += kStripe) {
                C a[kStripe];
#pragma unroll
                for (int q = 0; q < kStripe; q++)
                    if (i0 + q < n) a[q] = col[(long long)(i0 + q) * n];
#pragma unroll
                for (int q = 0; q < kStripe; q++) {
                    const int i = i0 + q;
                    if (i < n) {
                        a[q] = csub(a[q], cmul(y[i], vc));
                        col[(long long)i * n] = a[q];
                        if (i > k) s = cfma(CT<C>::mk(v[i].x, -v[i].y), a[q], s);
                    }
                }
            }
            const C wj = cmul(CT<C>::mk(tau.x, -tau.y), s);
            column_axpy(col, n, k + 1, n, v, CT<C>::mk(-wj.x, -wj.y));
        }
        // column k below the subdiagonal
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x)
            A[(long long)i * n + k] = (i == k + 1) ? s_beta : CT<C>::mk(0, 0);
        // Q[:, k+1:] -= (Q[:, k+1:] v) tau v^H
        __syncthreads();
        row_products(Q, v, y, n, k + 1, tau);
        __syncthreads();
        for (int j = k + 1 + threadIdx.x; j < n; j += blockDim.x)
            column_axpy(Q + j, n, 0, n, y, CT<C>::mk(-v[j].x, v[j].y));
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------
// The same reduction spread over the whole GPU: per column k three short launches for the
// batch -- the Householder vector (one CTA per matrix), the products y = tau A[:, k+1:] v and
// z = tau Q[:, k+1:] v (a warp per row, rows of every matrix over all SMs), and the updates of
// the columns k+1.. of A (right then left, one thread per column) and of Q.  Every element sees
// the operations of hessenberg_kernel in the same order; the kernel boundaries replace its
// block barriers, so the O(n^2) work of a column runs on every SM instead of one per matrix.
// Per matrix the 3n work entries hold v (slot 0: tau), y and z; ||A||_F^2 for the FP32 drop
// threshold ulp^2 ||A||_F^2 / n (||A||_F is invariant under the reduction) is kept in Q[n-1][0],
// which the reflectors never touch, and cleared at the end.
// ------------------------------------------------------------------------------------
constexpr int kHwRows = 8;        // rows (warps) per CTA of the product kernel
constexpr int kHwCols = 128;      // columns (threads) per CTA of the update kernel

template <typename C>
__global__ void __launch_bounds__(256) hw_init_kernel(C* __restrict__ Q, int n, long long sA, const int* __restrict__ skip) {
    if (skipped(skip, blockIdx.y)) return;
    Q += sA * blockIdx.y;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)n * n;
         i += (long long)gridDim.x * blockDim.x)
        Q[i] = CT<C>::mk((i / n) == (i % n) ? 1 : 0, 0);
}

// ||A||_F^2 into Q[n-1][0].x (after hw_init_kernel)
template <typename C>
__global__ void __launch_bounds__(256) hw_fro_kernel(const C* __restrict__ A, C* __restrict__ Q, int n, long long sA,
                                                     const int* __restrict__ skip) {
    using R = typename CT<C>::R;
    if (skipped(skip, blockIdx.y)) return;
    A += sA * blockIdx.y;
    __shared__ R sh[32];
    R a2 = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)n * n;
         i += (long long)gridDim.x * blockDim.x)
        a2 += cabs2(A[i]);
    a2 = block_sum(a2, sh);
    if (threadIdx.x == 0) atomicAdd(&Q[sA * blockIdx.y + (long long)(n - 1) * n].x, a2);
}

template <typename C>
__global__ void __launch_bounds__(256) hw_vec_kernel(C* __restrict__ A, const C* __restrict__ Q, int n, long long sA,
                                                     C* __restrict__ work, int k, const int* __restrict__ skip) {
    using R = typename CT<C>::R;
    if (skipped(skip, blockIdx.x)) return;
    A += sA * blockIdx.x;
    C* v = work + (long long)blockIdx.x * 3 * n;
    __shared__ R sh[32];
    __shared__ C s_beta;
    __shared__ int s_skip;
    constexpr bool kDropNegligible = sizeof(R) == sizeof(float);
    R xn2 = 0;
    for (int i = k + 2 + threadIdx.x; i < n; i += blockDim.x) xn2 += cabs2(A[(long long)i * n + k]);
    xn2 = block_sum(xn2, sh);
    const C alpha = A[(long long)(k + 1) * n + k];
    if (threadIdx.x == 0) {
        s_skip = 0;
        const R neg2 =
            kDropNegligible ? Q[sA * blockIdx.x + (long long)(n - 1) * n].x * CT<C>::ulp * CT<C>::ulp / (R)n : R(0);
        if (kDropNegligible && xn2 + cabs2(alpha) <= neg2) {
            s_skip = 2;                       // drop: zero the column below the diagonal
        } else if (xn2 == 0 && alpha.y == 0) {
            s_skip = 1;                       // already reduced
        } else {
            const R beta = -r_copysign(r_sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
            v[0] = CT<C>::mk((beta - alpha.x) / beta, -alpha.y / beta);      // tau
            s_beta = CT<C>::mk(beta, 0);
        }
        if (s_skip) v[0] = CT<C>::mk(0, 0);
    }
    __syncthreads();
    if (s_skip == 1) return;
    if (s_skip == 2) {
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[(long long)i * n + k] = CT<C>::mk(0, 0);
        return;
    }
    const C scal = cdiv(CT<C>::mk(1, 0), csub(alpha, s_beta));
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) {
        v[i] = (i == k + 1) ? CT<C>::mk(1, 0) : cmul(A[(long long)i * n + k], scal);
        A[(long long)i * n + k] = (i == k + 1) ? s_beta : CT<C>::mk(0, 0);
    }
}

// rows 0..n-1: y[i] = tau sum_{j > k} A[i][j] v[j]; rows n..2n-1: z[i] = tau sum_{j > k} Q[i][j] v[j]
template <typename C>
__global__ void __launch_bounds__(kHwRows * 32) hw_prod_kernel(const C* __restrict__ A, const C* __restrict__ Q, int n,
                                                               long long sA, C* __restrict__ work, int k,
                                                               const int* __restrict__ skip) {
    if (skipped(skip, blockIdx.y)) return;
    C* v = work + (long long)blockIdx.y * 3 * n;
    const C tau = v[0];
    if (tau.x == 0 && tau.y == 0) return;
    const int lane = threadIdx.x & 31;
    const int r = blockIdx.x * kHwRows + (threadIdx.x >> 5);
    if (r >= 2 * n) return;
    const C* row = (r < n ? A + (long long)r * n : Q + (long long)(r - n) * n) + sA * blockIdx.y;
    C acc = CT<C>::mk(0, 0);
#pragma unroll 4
    for (int j = k + 1 + lane; j < n; j += 32) acc = cfma(row[j], v[j], acc);
    for (int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
    if (lane == 0) v[n + r] = cmul(tau, acc);          // y = v + n, z = v + 2n
}

// columns j > k of A: right update (all rows) while summing v^H of the updated column, then the
// left update; columns j > k of Q (blocks past the A blocks): Q[:, j] -= z conj(v_j)
template <typename C>
__global__ void __launch_bounds__(kHwCols) hw_update_kernel(C* __restrict__ A, C* __restrict__ Q, int n, long long sA,
                                                            const C* __restrict__ work, int k, int nblk_a,
                                                            const int* __restrict__ skip) {
    if (skipped(skip, blockIdx.y)) return;
    const C* v = work + (long long)blockIdx.y * 3 * n;
    const C tau = v[0];
    if (tau.x == 0 && tau.y == 0) return;
    constexpr int kStripe = sizeof(typename CT<C>::R) == sizeof(float) ? 8 : 4;
    const bool isA = (int)blockIdx.x < nblk_a;
    const int j = k + 1 + (isA ? (int)blockIdx.x : (int)blockIdx.x - nblk_a) * kHwCols + threadIdx.x;
    if (j >= n) return;
    if (isA) {
        const C* y = v + n;
        const C vc = CT<C>::mk(v[j].x, -v[j].y);
        C* col = A + sA * blockIdx.y + j;
        C s = CT<C>::mk(0, 0);
        for (int i0 = 0; i0 < n; i0 += kStripe) {
            C a[kStripe];
#pragma unroll
            for (int q = 0; q < kStripe; q++)
                if (i0 + q < n) a[q] = col[(long long)(i0 + q) * n];
#pragma unroll
            for (int q = 0; q < kStripe; q++) {
                const int i = i0 + q;
                if (i < n) {
                    a[q] = csub(a[q], cmul(y[i], vc));
                    col[(long long)i * n] = a[q];
                    if (i > k) s = cfma(CT<C>::mk(v[i].x, -v[i].y), a[q], s);
                }
            }
        }
        const C wj = cmul(CT<C>::mk(tau.x, -tau.y), s);
        column_axpy(col, n, k + 1, n, v, CT<C>::mk(-wj.x, -wj.y));
    } else {
        column_axpy(Q + sA * blockIdx.y + j, n, 0, n, v + 2 * n, CT<C>::mk(-v[j].x, v[j].y));
    }
}

template <typename C>
__global__ void hw_finish_kernel(C* __restrict__ Q, int n, long long sA, int batch, const int* __restrict__ skip) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < batch && !skipped(skip, b)) Q[sA * b + (long long)(n - 1) * n] = CT<C>::mk(0, 0);
}

// ------------------------------------------------------------------------------------
// Single-shift complex QR (zlahqr semantics: wantt, wantz) on the upper Hessenberg H with
// Schur vectors accumulated into Z (Z := Z G^H).  One CTA per matrix.  status[b]: 0 ok,
// 1 no convergence within 30 n iterations.
// ------------------------------------------------------------------------------------
// G [x; y] (rows) and [x, y] G^H (columns) for G = [c, s; -conj(s), c]
template <typename C>
__device__ __forceinline__ void rot_rows(typename CT<C>::R c, C s, C& x, C& y) {
    const C nx = CT<C>::mk(c * x.x + (s.x * y.x - s.y * y.y), c * x.y + (s.x * y.y + s.y * y.x));
    const C ny = CT<C>::mk(c * y.x - (s.x * x.x + s.y * x.y), c * y.y - (s.x * x.y - s.y * x.x));
    x = nx;
    y = ny;
}
template <typename C>
__device__ __forceinline__ void rot_cols(typename CT<C>::R c, C s, C& x, C& y) {
    const C nx = CT<C>::mk(c * x.x + (y.x * s.x + y.y * s.y), c * x.y + (y.y * s.x - y.x * s.y));
    const C ny = CT<C>::mk(c * y.x - (x.x * s.x - x.y * s.y), c * y.y - (x.x * s.y + x.y * s.x));
    x = nx;
    y = ny;
}

// Rotations k0 .. k1-1 of a single-shift sweep over the active block [l, ihi].  Rotation k
// touches rows / columns k, k+1 only, so the chase needs just the window rows k0..k1+1,
// columns k0-1..k1: warp 0 runs it in shared memory (one rotation after another, no block
// barrier) and records the rotations.  Then the whole CTA applies them, in order, to what lies
// outside the window: rows k0..k1 right of column k1, columns k0..k1 above row k0, and the
// Schur vectors Z[:, k0..k1], each thread streaming one column or row with two values live.
// Every element sees the same operations in the same order as rotation-by-rotation.
constexpr int kHqrW = 64;

// Givens generator of the chase, from two reciprocal square roots (c = |f| / d,
// s = conj(g) f / (|f| d), r = f d / |f| with d = sqrt(|f|^2 + |g|^2)), which keeps the rotation
// unitary to a few ulp.  In FP64 this replaces zlartg's two square roots and five divisions:
// the chase is one warp working through each rotation's dependent chain, and GB300 issues FP64
// at about 2 operations per clock per SM, so that chain sets the FP64 sweep's time.  (In FP32,
// one Newton-Raphson step on each reciprocal square root, unitary to about 1 ulp, was measured on
// two n = 3200 layers: eigenpair residuals 1.6-2.5x larger and fewer layers accepted by the
// refinement, so the plain form stays.)
__device__ __forceinline__ float r_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double r_rsqrt(double x) { return rsqrt(x); }

template <typename C>
__device__ __forceinline__ void givens_chase(C f, C g, typename CT<C>::R& c, C& s, C& r) {
    using R = typename CT<C>::R;
    const R gf = cabs2(g), ff = cabs2(f);
    if (gf == R(0)) {
        c = R(1);
        s = CT<C>::mk(R(0), R(0));
        r = f;
        return;
    }
    if (ff == R(0)) {
        const R ig = r_rsqrt(gf);
        c = R(0);
        s = CT<C>::mk(g.x * ig, -g.y * ig);
        r = CT<C>::mk(gf * ig, R(0));
        return;
    }
    const R iaf = r_rsqrt(ff), id = r_rsqrt(ff + gf);
    c = ff * iaf * id;
    const C fs = CT<C>::mk(f.x * iaf, f.y * iaf);
    const C t = cmulc(g, fs);
    s = CT<C>::mk(t.x * id, t.y * id);
    const R d = (ff + gf) * id;
    r = CT<C>::mk(fs.x * d, fs.y * d);
}

// The chase of rotations k0 .. k1-1 inside the shared-memory window (loaded from H, a block
// barrier, the chase by warp 0, a block barrier, stored back), the rotations recorded in hc / hs.
template <typename C, bool kCg>
__device__ void hqr_chase(C* __restrict__ H, int n, int l, int ihi, int k0, int k1, C shift, C* hw,
                          typename CT<C>::R* hc, C* hs) {
    using R = typename CT<C>::R;
    constexpr int ldw = kHqrW + 2;
    const int r1 = min(k1 + 1, ihi);
    const int c0 = (k0 > l) ? k0 - 1 : k0;
    const int nr = r1 - k0 + 1, nc = k1 - c0 + 1;
    for (int e = threadIdx.x; e < nr * nc; e += blockDim.x) {
        const int i = e / nc, j = e % nc;
        hw[i * ldw + j] = hld<kCg>(H + (long long)(k0 + i) * n + c0 + j);
    }
    __syncthreads();
#define HW(i, j) hw[((i) - k0) * ldw + ((j) - c0)]
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        for (int k = k0; k < k1; k++) {
            // every lane generates the rotation (no broadcast needed); lane 0 records it
            C f, g, r, s;
            R c;
            if (k == l) {
                f = csub(HW(l, l), shift);
                g = HW(l + 1, l);
            } else {
                f = HW(k, k - 1);
                g = HW(k + 1, k - 1);
            }
            givens_chase(f, g, c, s, r);
            __syncwarp();
            if (lane == 0) {
                if (k > l) {
                    HW(k, k - 1) = r;
                    HW(k + 1, k - 1) = CT<C>::mk(0, 0);
                }
                hc[k - k0] = c;
                hs[k - k0] = s;
            }
            for (int j = k + lane; j <= k1; j += 32) rot_rows(c, s, HW(k, j), HW(k + 1, j));
            __syncwarp();
            const int rmax = min(k + 2, ihi);
            for (int i = k0 + lane; i <= rmax; i += 32) rot_cols(c, s, HW(i, k), HW(i, k + 1));
            __syncwarp();
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nr * nc; e += blockDim.x) {
        const int i = e / nc, j = e % nc;
        H[(long long)(k0 + i) * n + c0 + j] = hw[i * ldw + j];
    }
#undef HW
}

// The recorded rotations applied, in order, to what lies outside the window: tasks t0, t0 + dt,
// ... of the stripes (columns right of the window, rows above it, Schur-vector rows).  Each task
// streams one stripe of k1 - k0 + 1 values.  The values are loaded kStripe at a time into
// registers before the rotations run through them: a load-rotate-store chain per element would
// wait a full memory latency per element (the compiler cannot move a load of the stripe above the
// store to the element before it).
template <typename C, bool kCg>
__device__ void hqr_apply(C* __restrict__ H, C* __restrict__ Z, int n, int k0, int k1, const typename CT<C>::R* hc,
                          const C* hs, int t0, int dt) {
    using R = typename CT<C>::R;
    constexpr int kStripe = sizeof(R) == sizeof(float) ? 16 : 4;
    const int nright = n - 1 - k1, nabove = k0;
    for (int t = t0; t < nright + nabove + n; t += dt) {
        const bool right = t < nright;              // column j (rows k0..k1), else a row (columns k0..k1)
        C* base;
        long long step;
        if (right) {
            base = H + k1 + 1 + t;
            step = n;
        } else {
            base = (t < nright + nabove) ? H + (long long)(t - nright) * n : Z + (long long)(t - nright - nabove) * n;
            step = 1;
        }
        C x = hld<kCg>(base + (long long)k0 * step);
        for (int kb = k0; kb < k1; kb += kStripe) {
            const int m = min(kStripe, k1 - kb);
            C y[kStripe];
#pragma unroll
            for (int q = 0; q < kStripe; q++)
                if (q < m) y[q] = hld<kCg>(base + (long long)(kb + q + 1) * step);
#pragma unroll
            for (int q = 0; q < kStripe; q++) {
                if (q < m) {
                    if (right)
                        rot_rows(hc[kb + q - k0], hs[kb + q - k0], x, y[q]);
                    else
                        rot_cols(hc[kb + q - k0], hs[kb + q - k0], x, y[q]);
                    base[(long long)(kb + q) * step] = x;
                    x = y[q];
                }
            }
        }
        base[(long long)k1 * step] = x;
    }
}

template <typename C>
__device__ void hqr_chunk(C* __restrict__ H, C* __restrict__ Z, int n, int l, int ihi, int k0, int k1, C shift,
                          C* hw, typename CT<C>::R* hc, C* hs) {
    hqr_chase<C, false>(H, n, l, ihi, k0, k1, shift, hw, hc, hs);
    hqr_apply<C, false>(H, Z, n, k0, k1, hc, hs, threadIdx.x, blockDim.x);
    __syncthreads();
}

// Shift of the next sweep over [l, ihi]: Wilkinson's from the trailing 2 x 2 block, and
// exceptional shifts every 10 iterations without a deflation (zlahqr's KEXSH rule).
template <typename C, bool kCg>
__device__ C hqr_shift(const C* __restrict__ H, int n, int l, int ihi, int its) {
    using R = typename CT<C>::R;
    const C hii = hld<kCg>(H + (long long)ihi * n + ihi);
    if (its % 20 == 0) return CT<C>::mk(R(0.75) * r_abs(hld<kCg>(H + (long long)ihi * n + ihi - 1).x) + hii.x, hii.y);
    if (its % 10 == 0) {
        const C hll = hld<kCg>(H + (long long)l * n + l);
        return CT<C>::mk(R(0.75) * r_abs(hld<kCg>(H + (long long)(l + 1) * n + l).x) + hll.x, hll.y);
    }
    const C a = hld<kCg>(H + (long long)(ihi - 1) * n + ihi - 1);
    const C b = hld<kCg>(H + (long long)(ihi - 1) * n + ihi);
    const C c = hld<kCg>(H + (long long)ihi * n + ihi - 1);
    const C d = hii;
    const C half = CT<C>::mk(R(0.5) * (a.x - d.x), R(0.5) * (a.y - d.y));
    const C bc = cmul(b, c);
    const C disc = cfma(half, half, bc);
    const C sq = zsqrt(disc);
    // choose the root that makes the shift closer to d
    C e1 = cadd(half, sq), e2 = csub(half, sq);
    const C den = cabs2(e1) >= cabs2(e2) ? e1 : e2;
    return (cabs2(den) == 0) ? d : csub(d, cdiv(bc, den));
}

template <typename C>
constexpr size_t hqr_smem_bytes() {
    return sizeof(C) * ((kHqrW + 2) * (kHqrW + 2) + kHqrW) + sizeof(typename CT<C>::R) * kHqrW;
}

template <typename C>
__global__ void __launch_bounds__(1024)
hqr_kernel(C* __restrict__ H, C* __restrict__ Z, int n, long long sA, C* __restrict__ eig, int* __restrict__ status,
           const int* __restrict__ skip) {
    using R = typename CT<C>::R;
    if (skipped(skip, blockIdx.x)) return;
    H += sA * blockIdx.x;
    Z += sA * blockIdx.x;
    eig += (long long)n * blockIdx.x;
    __shared__ C s_s;
    __shared__ int s_red[32];
    extern __shared__ __align__(16) unsigned char hqr_smem[];
    C* hw = reinterpret_cast<C*>(hqr_smem);                         // (kHqrW + 2)^2 window
    C* hs = hw + (kHqrW + 2) * (kHqrW + 2);                         // kHqrW rotation sines
    R* hc = reinterpret_cast<R*>(hs + kHqrW);                       // kHqrW rotation cosines
    int ihi = n - 1;
    int its = 0;
    const int itmax = 30 * max(10, n);
    int total = 0;
    while (ihi >= 0) {
        // the largest k in [1, ihi] whose subdiagonal entry may be set to zero (0: none);
        // each thread scans its ks downwards, then a block maximum
        int lk = 0;
        for (int k = ihi - (int)threadIdx.x; k > 0; k -= blockDim.x)
            if (hqr_deflates(H, n, k, ihi)) {
                lk = k;
                break;
            }
        lk = __reduce_max_sync(0xffffffffu, lk);
        if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = lk;
        __syncthreads();
        int l = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) l = max(l, s_red[w]);
        __syncthreads();
        if (l > 0) {
            if (threadIdx.x == 0) H[(long long)l * n + l - 1] = CT<C>::mk(0, 0);
        }
        if (l >= ihi) {                                   // 1x1 block: eigenvalue converged
            if (threadIdx.x == 0) eig[ihi] = H[(long long)ihi * n + ihi];
            __syncthreads();
            ihi = l - 1;
            its = 0;
            continue;
        }
        if (total > itmax) {
            if (threadIdx.x == 0) status[blockIdx.x] = 1;
            return;
        }
        its++;
        total++;
        // shift; exceptional shifts every 10 iterations without a deflation (zlahqr's KEXSH rule)
        if (threadIdx.x == 0) s_s = hqr_shift<C, false>(H, n, l, ihi, its);
        __syncthreads();
        const C shift = s_s;
        __syncthreads();
        // implicit single-shift QR sweep over the active block [l, ihi], kHqrW rotations at a time
        for (int k0 = l; k0 < ihi; k0 += kHqrW) {
            const int k1 = min(k0 + kHqrW, ihi);
            hqr_chunk(H, Z, n, l, ihi, k0, k1, shift, hw, hc, hs);
        }
    }
}

// ------------------------------------------------------------------------------------
// The same QR with each matrix on a thread-block cluster of K CTAs (K = the cluster size, 2..8):
// rank 0 makes every decision (deflations, shift, end) and chases each window as hqr_kernel does;
// after a cluster barrier every CTA copies the window's rotations from rank 0's shared memory and
// applies them to its share of the stripes (task t to CTA t / blockDim mod K), then a second
// barrier.  The CTAs follow the decisions rank 0 leaves in its shared memory before a barrier,
// so all of them pass the same sequence of barriers and leave together.  H and Z are read through
// L2 only (other CTAs of the cluster write them) and every thread fences its writes before a
// barrier.  Each element sees the same rotations in the same order as in hqr_kernel; the two
// kernels are compiled apart and may fuse multiply-adds differently, so the results agree to
// rounding (measured: they differ in the last bits even where the second CTA has no stripe to
// update).  The deferred updates, 72-80 % of a sweep on one CTA (and nearly all of it in FP64,
// whose rate per SM is low), are spread over K SMs.
// ------------------------------------------------------------------------------------
template <typename C>
__global__ void __launch_bounds__(1024)
hqr_cluster_kernel(C* __restrict__ H, C* __restrict__ Z, int n, long long sA, C* __restrict__ eig,
                   int* __restrict__ status, const int* __restrict__ skip) {
    using R = typename CT<C>::R;
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int K = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int b = blockIdx.x / K;
    if (skipped(skip, b)) return;                       // the whole cluster, before any barrier
    H += sA * b;
    Z += sA * b;
    eig += (long long)n * b;
    __shared__ C s_shift;
    __shared__ int s_red[32];
    __shared__ int s_cmd[3];                            // rank 0: operation (0 sweep, 1 end), l, ihi
    extern __shared__ __align__(16) unsigned char hqr_smem[];
    C* hw = reinterpret_cast<C*>(hqr_smem);
    C* hs = hw + (kHqrW + 2) * (kHqrW + 2);
    R* hc = reinterpret_cast<R*>(hs + kHqrW);
    const int* cmd0 = cluster.map_shared_rank(s_cmd, 0);
    const C* hs0 = cluster.map_shared_rank(hs, 0);
    const R* hc0 = cluster.map_shared_rank(hc, 0);
    int ihi = n - 1;                                    // rank 0's state
    int its = 0;
    const int itmax = 30 * max(10, n);
    int total = 0;
    while (true) {
        if (rank == 0) {
            // deflations until a sweep is due, the matrix is done or the iteration limit is hit
            int op = 0, l = 0;
            while (true) {
                if (ihi < 0) {
                    op = 1;
                    break;
                }
                int lk = 0;
                for (int k = ihi - (int)threadIdx.x; k > 0; k -= blockDim.x)
                    if (hqr_deflates<C, true>(H, n, k, ihi)) {
                        lk = k;
                        break;
                    }
                lk = __reduce_max_sync(0xffffffffu, lk);
                if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = lk;
                __syncthreads();
                l = 0;
                for (int w = 0; w < (int)(blockDim.x >> 5); w++) l = max(l, s_red[w]);
                __syncthreads();
                if (l > 0 && threadIdx.x == 0) H[(long long)l * n + l - 1] = CT<C>::mk(0, 0);
                if (l >= ihi) {                           // 1x1 block: eigenvalue converged
                    if (threadIdx.x == 0) eig[ihi] = hld<true>(H + (long long)ihi * n + ihi);
                    __syncthreads();
                    ihi = l - 1;
                    its = 0;
                    continue;
                }
                if (total > itmax) {
                    if (threadIdx.x == 0) status[b] = 1;
                    op = 1;
                    break;
                }
                its++;
                total++;
                if (threadIdx.x == 0) s_shift = hqr_shift<C, true>(H, n, l, ihi, its);
                break;
            }
            if (threadIdx.x == 0) {
                s_cmd[0] = op;
                s_cmd[1] = l;
                s_cmd[2] = ihi;
            }
        }
        __threadfence();
        cluster.sync();
        const int op = cmd0[0], l = cmd0[1], hi = cmd0[2];
        if (op != 0) {
            cluster.sync();                              // rank 0's shared memory stays until all have read
            return;
        }
        // implicit single-shift QR sweep over [l, hi], kHqrW rotations at a time (l < hi)
        for (int k0 = l; k0 < hi; k0 += kHqrW) {
            const int k1 = min(k0 + kHqrW, hi);
            if (rank == 0) hqr_chase<C, true>(H, n, l, hi, k0, k1, s_shift, hw, hc, hs);
            __threadfence();
            cluster.sync();
            if (rank != 0) {
                for (int i = threadIdx.x; i < k1 - k0; i += blockDim.x) {
                    hc[i] = hc0[i];
                    hs[i] = hs0[i];
                }
                __syncthreads();
            }
            hqr_apply<C, true>(H, Z, n, k0, k1, hc, hs, rank * (int)blockDim.x + (int)threadIdx.x,
                               K * (int)blockDim.x);
            __threadfence();
            cluster.sync();
        }
    }
}

// ------------------------------------------------------------------------------------
// Eigenvectors of the upper triangular Schur factor T (ztrevc semantics, right vectors):
// X[:, k] solves (T - T_kk I) x = 0 with x_k = 1, x_i = 0 for i > k.  One warp per vector.
// X is written row-major (column k = eigenvector k).
// FP64: a denominator T_ii - T_kk below smin is replaced by smin, as ztrevc does.  FP32 (the
// first stage of the mixed solver): where both the denominator and the coupling sum
// sum_j T_ij x_j are within 16 ulp of max |T_jj|, the pair counts as one degenerate eigenvalue and
// x_i = 0, so each keeps its own Schur vector.  (Dividing rounding noise by rounding noise gives
// numerically parallel vectors for the exactly degenerate eigenvalues of homogeneous layers; the
// refinement resolves such clusters in FP64.)  A close pair with a real coupling is divided as in
// FP64: zeroing it would leave the coupling as residual, which the refinement of dense spectra
// (n = 3200 layers) could not remove.
// ------------------------------------------------------------------------------------
template <typename C>
__global__ void __launch_bounds__(256)
trevc_kernel(const C* __restrict__ T, C* __restrict__ X, int n, long long sA, const int* __restrict__ skip) {
    using R = typename CT<C>::R;
    constexpr bool kDegenerateSkip = sizeof(R) == sizeof(float);
    if (skipped(skip, blockIdx.y)) return;
    T += sA * blockIdx.y;
    X += sA * blockIdx.y;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n) return;
    const int k = warp;
    const R ulp = CT<C>::ulp;
    const C lam = T[(long long)k * n + k];
    const R smin = r_max(ulp * cabs1(lam), CT<C>::safmin * ((R)n / ulp));
    R deg = 0;
    if (kDegenerateSkip) {
        for (int i = lane; i < n; i += 32) deg = r_max(deg, cabs1(T[(long long)i * n + i]));
        for (int o = 16; o > 0; o >>= 1) deg = r_max(deg, __shfl_xor_sync(0xffffffffu, deg, o));
        deg *= R(16) * ulp;
    }
    // x_k = 1, x_{k+1..} = 0
    for (int i = lane; i < n; i += 32) X[(long long)i * n + k] = CT<C>::mk(i == k ? 1 : 0, 0);
    __syncwarp();
    for (int i = k - 1; i >= 0; i--) {
        // x_i = -(sum_{j=i+1..k} T_ij x_j) / (T_ii - lam)
        C s = CT<C>::mk(0, 0);
        for (int j = i + 1 + lane; j <= k; j += 32) s = cfma(T[(long long)i * n + j], X[(long long)j * n + k], s);
        for (int o = 16; o > 0; o >>= 1) {
            s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
            s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
        }
        if (lane == 0) {
            C d = csub(T[(long long)i * n + i], lam);
            if (kDegenerateSkip && cabs1(d) <= deg && cabs1(s) <= deg) {
                X[(long long)i * n + k] = CT<C>::mk(0, 0);
            } else {
                if (cabs1(d) < smin) d = CT<C>::mk(smin, 0);
                X[(long long)i * n + k] = cdiv(CT<C>::mk(-s.x, -s.y), d);
            }
        }
        __syncwarp();
    }
}

// copy of the batch entries that are not skipped
template <typename C>
__global__ void copy_kernel(const C* __restrict__ src, C* __restrict__ dst, long long count, const int* __restrict__ skip) {
    if (skipped(skip, blockIdx.y)) return;
    src += count * blockIdx.y;
    dst += count * blockIdx.y;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

}  // namespace z

// ------------------------------------------------------------------------------------
// Host wrappers
// ------------------------------------------------------------------------------------
template <typename C>
scw_status gemm(cudaStream_t st, int M, int N, int K, C alpha, const C* A, int lda, long long sA, const C* B, int ldb,
                long long sB, C beta, C* Cm, int ldc, long long sC, int batch, const int* skip) {
    if (M <= 0 || N <= 0 || batch <= 0) return SCW_OK;
    dim3 grid((N + z::kGT - 1) / z::kGT, (M + z::kGT - 1) / z::kGT, batch);
    z::gemm_kernel<C><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, Cm, ldc, sC, skip);
    SCW_CUDA_TRY(cudaGetLastError());
    return SCW_OK;
}

template <typename C>
scw_status getrf(cudaStream_t st, C* A, int n, long long sA, int* piv, long long sP, int* info, int batch) {
    if (n <= 0 || batch <= 0) return SCW_OK;
    SCW_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(int) * batch, st));
    const C one = {1, 0}, minus = {-1, 0};
    for (int k0 = 0; k0 < n; k0 += z::kNB) {
        const int nb = std::min(z::kNB, n - k0);
        z::lu_panel_kernel<C><<<batch, 512, 0, st>>>(A, n, n, sA, k0, nb, piv, sP, info);
        SCW_CUDA_TRY(cudaGetLastError());
        dim3 g2((n + 255) / 256, batch);
        z::lu_swap_trsm_kernel<C><<<g2, 256, 0, st>>>(A, n, n, sA, k0, nb, piv, sP);
        SCW_CUDA_TRY(cudaGetLastError());
        const int rem = n - k0 - nb;
        if (rem > 0) {
            // A22 -= L21 U12
            scw_status s = gemm<C>(st, rem, rem, nb, minus, A + (long long)(k0 + nb) * n + k0, n, sA,
                                   A + (long long)k0 * n + k0 + nb, n, sA, one, A + (long long)(k0 + nb) * n + k0 + nb,
                                   n, sA, batch);
            if (s != SCW_OK) return s;
        }
    }
    return SCW_OK;
}

template <typename C>
scw_status getrs(cudaStream_t st, const C* LU, int n, long long sA, const int* piv, long long sP, C* B, int nrhs,
                 long long sB, int batch) {
    // blocked: per diagonal block a small triangular solve, the rest of the rows updated by GEMM
    if (n <= 0 || nrhs <= 0 || batch <= 0) return SCW_OK;
    constexpr int kTB = 64;
    const C one = {1, 0}, minus = {-1, 0};
    const dim3 g((nrhs + 255) / 256, batch);
    z::laswp_kernel<C><<<g, 256, 0, st>>>(piv, sP, B, nrhs, sB, n, nrhs);
    SCW_CUDA_TRY(cudaGetLastError());
    for (int k0 = 0; k0 < n; k0 += kTB) {
        const int nb = std::min(kTB, n - k0);
        z::trsm_block_kernel<C><<<g, 256, 0, st>>>(LU, n, sA, k0, nb, B, nrhs, sB, nrhs, 0);
        SCW_CUDA_TRY(cudaGetLastError());
        const int rem = n - k0 - nb;
        if (rem > 0) {
            scw_status s = gemm<C>(st, rem, nrhs, nb, minus, LU + (long long)(k0 + nb) * n + k0, n, sA,
                                   B + (long long)k0 * nrhs, nrhs, sB, one, B + (long long)(k0 + nb) * nrhs, nrhs, sB,
                                   batch);
            if (s != SCW_OK) return s;
        }
    }
    for (int k0 = ((n - 1) / kTB) * kTB; k0 >= 0; k0 -= kTB) {
        const int nb = std::min(kTB, n - k0);
        z::trsm_block_kernel<C><<<g, 256, 0, st>>>(LU, n, sA, k0, nb, B, nrhs, sB, nrhs, 1);
        SCW_CUDA_TRY(cudaGetLastError());
        if (k0 > 0) {
            scw_status s = gemm<C>(st, k0, nrhs, nb, minus, LU + k0, n, sA, B + (long long)k0 * nrhs, nrhs, sB, one, B,
                                   nrhs, sB, batch);
            if (s != SCW_OK) return s;
        }
    }
    return SCW_OK;
}

scw_status zgehrd(cudaStream_t st, double2* A, double2* Q, int n, int batch, double2* work) {
    if (n <= 0 || batch <= 0) return SCW_OK;
    z::hessenberg_kernel<double2><<<batch, 1024, 0, st>>>(A, Q, n, (long long)n * n, work, nullptr);
    SCW_CUDA_TRY(cudaGetLastError());
    return SCW_OK;
}

// Hessenberg reduction with Schur-vector accumulation, spread over the GPU (3 launches per column)
template <typename C>
static scw_status gehrd_wide(cudaStream_t st, C* A, C* Q, int n, int batch, C* hw, const int* skip) {
    const long long nn = (long long)n * n;
    const unsigned gi = (unsigned)std::min<long long>((nn + 255) / 256, 1024);
    z::hw_init_kernel<C><<<dim3(gi, batch), 256, 0, st>>>(Q, n, nn, skip);
    z::hw_fro_kernel<C><<<dim3(gi, batch), 256, 0, st>>>(A, Q, n, nn, skip);
    SCW_CUDA_TRY(cudaGetLastError());
    for (int k = 0; k + 2 < n; k++) {
        z::hw_vec_kernel<C><<<batch, 256, 0, st>>>(A, Q, n, nn, hw, k, skip);
        z::hw_prod_kernel<C><<<dim3((2 * n + z::kHwRows - 1) / z::kHwRows, batch), z::kHwRows * 32, 0, st>>>(
            A, Q, n, nn, hw, k, skip);
        const int nblk = (n - k - 1 + z::kHwCols - 1) / z::kHwCols;
        z::hw_update_kernel<C><<<dim3(2 * nblk, batch), z::kHwCols, 0, st>>>(A, Q, n, nn, hw, k, nblk, skip);
    }
    z::hw_finish_kernel<C><<<(batch + 255) / 256, 256, 0, st>>>(Q, n, nn, batch, skip);
    SCW_CUDA_TRY(cudaGetLastError());
    return SCW_OK;
}

// CTAs per matrix of the QR sweeps: 0 = chosen per call, 1 = one CTA (hqr_kernel), 2..8 = a
// cluster of that size (scw_set_qr_cluster)
static std::atomic<int> g_qr_cluster{0};

// The QR sweeps of `batch` matrices, `active` of them not skipped.  Single solves (wide) put each
// matrix on a cluster of K CTAs: the largest K <= 8 for which all active matrices' clusters are
// resident at once (cudaOccupancyMaxActiveClusters) and, in FP32, no larger than the stripes of a
// window fill (2n tasks for K x 1024 threads; FP64 updates are bound by the FP64 rate of each SM
// and gain from more SMs down to fewer tasks per CTA).  Otherwise one CTA per matrix.
template <typename C>
static scw_status hqr_launch(cudaStream_t st, C* A, C* Q, int n, long long nn, C* W, int* status, const int* skip,
                             int batch, int active, bool wide) {
    const size_t smem = z::hqr_smem_bytes<C>();
    const int force = g_qr_cluster.load();
    if (wide && force != 1 && active > 0) {
        int dev = 0, sms = 0;
        SCW_CUDA_TRY(cudaGetDevice(&dev));
        SCW_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        SCW_CUDA_TRY(cudaFuncSetAttribute(z::hqr_cluster_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        int kmax = force > 1 ? std::min(force, 8) : std::min(8, sms / active);
        if (force <= 1 && sizeof(C) == sizeof(float2)) kmax = std::min(kmax, (2 * n + 1023) / 1024);
        for (int k = kmax; k >= 2; k--) {
            cudaLaunchConfig_t cfg = {};
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = (unsigned)k;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.gridDim = dim3((unsigned)(k * batch));
            cfg.blockDim = dim3(1024);
            cfg.dynamicSmemBytes = smem;
            cfg.stream = st;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int resident = 0;
            if (cudaOccupancyMaxActiveClusters(&resident, z::hqr_cluster_kernel<C>, &cfg) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            if (resident >= (force > 1 ? 1 : active)) {
                SCW_CUDA_TRY(cudaLaunchKernelEx(&cfg, z::hqr_cluster_kernel<C>, A, Q, n, nn, W, status, skip));
                return SCW_OK;
            }
        }
    }
    SCW_CUDA_TRY(cudaFuncSetAttribute(z::hqr_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    z::hqr_kernel<C><<<batch, 1024, smem, st>>>(A, Q, n, nn, W, status, skip);
    SCW_CUDA_TRY(cudaGetLastError());
    return SCW_OK;
}

template <typename C>
scw_status geev(cudaStream_t st, C* A, C* W, C* V, int n, int batch, C* work, int* status, const int* skip,
                bool wide) {
    // A (overwritten): n x n per batch entry; W: n eigenvalues; V: n x n right eigenvectors (columns)
    // work: >= batch * (n*n + 3 n) elements
    if (n <= 0 || batch <= 0) return SCW_OK;
    const long long nn = (long long)n * n;
    C* Q = work;                             // batch * n * n: Schur vectors
    C* hw = work + nn * batch;               // batch * 3n
    SCW_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int) * batch, st));
    // single solves outside a stream capture count the matrices the skip mask leaves (and do
    // nothing when it leaves none)
    int active = batch;
    if (wide && skip) {
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        SCW_CUDA_TRY(cudaStreamIsCapturing(st, &cap));
        if (cap == cudaStreamCaptureStatusNone) {
            std::vector<int> sk(batch);
            SCW_CUDA_TRY(cudaMemcpyAsync(sk.data(), skip, sizeof(int) * batch, cudaMemcpyDeviceToHost, st));
            SCW_CUDA_TRY(cudaStreamSynchronize(st));
            active = (int)std::count(sk.begin(), sk.end(), 0);
            if (active == 0) return SCW_OK;
        }
    }
    if (wide && n >= kWideMinN) {
        scw_status s = gehrd_wide<C>(st, A, Q, n, batch, hw, skip);
        if (s != SCW_OK) return s;
    } else {
        z::hessenberg_kernel<C><<<batch, 1024, 0, st>>>(A, Q, n, nn, hw, skip);
        SCW_CUDA_TRY(cudaGetLastError());
    }
    {
        scw_status s = hqr_launch<C>(st, A, Q, n, nn, W, status, skip, batch, active, wide);
        if (s != SCW_OK) return s;
    }
    // X (triangular eigenvectors) into V, then A := Q X, copied to V
    dim3 gt((n * 32 + 255) / 256, batch);
    z::trevc_kernel<C><<<gt, 256, 0, st>>>(A, V, n, nn, skip);
    SCW_CUDA_TRY(cudaGetLastError());
    const C one = {1, 0}, zero = {0, 0};
    scw_status s = gemm<C>(st, n, n, n, one, Q, n, nn, V, n, nn, zero, A, n, nn, batch, skip);
    if (s != SCW_OK) return s;
    z::copy_kernel<C><<<dim3((unsigned)std::min<long long>((nn + 255) / 256, 4096), batch), 256, 0, st>>>(A, V, nn, skip);
    SCW_CUDA_TRY(cudaGetLastError());
    return SCW_OK;
}

#define SCW_DENSE_INSTANTIATE(C)                                                                                    \
    template scw_status gemm<C>(cudaStream_t, int, int, int, C, const C*, int, long long, const C*, int, long long, \
                                C, C*, int, long long, int, const int*);                                           \
    template scw_status getrf<C>(cudaStream_t, C*, int, long long, int*, long long, int*, int);                    \
    template scw_status getrs<C>(cudaStream_t, const C*, int, long long, const int*, long long, C*, int, long long, \
                                 int);                                                                             \
    template scw_status geev<C>(cudaStream_t, C*, C*, C*, int, int, C*, int*, const int*, bool);
SCW_DENSE_INSTANTIATE(double2)
SCW_DENSE_INSTANTIATE(float2)
#undef SCW_DENSE_INSTANTIATE

}  // namespace scw

// ------------------------------------------------------------------------------------
// C ABI: GPU replacements of the reference's LAPACK wrappers (third_Lapack.h:38-87), on
// device buffers, batched.
// ------------------------------------------------------------------------------------
using scw::fail;

extern "C" {

scw_status scw_zgemm(scw_ctx ctx, int M, int N, int K, const double* alpha, const void* A, const void* B,
                     const double* beta, void* C, int batch) {
    if (!ctx || !A || !B || !C || !alpha || !beta || M < 0 || N < 0 || K < 0 || batch < 1)
        return fail(SCW_ERR_ARG, "scw_zgemm: bad arguments");
    SCW_ON_DEVICE(ctx->device);
    ctx->launches++;
    return scw::zgemm(ctx->stream, M, N, K, make_double2(alpha[0], alpha[1]), (const double2*)A, K, (long long)M * K,
                      (const double2*)B, N, (long long)K * N, make_double2(beta[0], beta[1]), (double2*)C, N,
                      (long long)M * N, batch);
}

scw_status scw_zgesv(scw_ctx ctx, int n, int nrhs, void* A, void* B, int batch, int* info_host) {
    if (!ctx || !A || !B || n < 1 || nrhs < 1 || batch < 1) return fail(SCW_ERR_ARG, "scw_zgesv: bad arguments");
    SCW_ON_DEVICE(ctx->device);
    int* dpiv = nullptr;
    int* dinfo = nullptr;
    if (cudaMalloc(&dpiv, sizeof(int) * (size_t)n * batch) != cudaSuccess ||
        cudaMalloc(&dinfo, sizeof(int) * (size_t)batch) != cudaSuccess) {
        cudaFree(dpiv);
        return fail(SCW_ERR_NOMEM, "scw_zgesv: pivots");
    }
    const long long nn = (long long)n * n;
    scw_status st = scw::zgetrf(ctx->stream, (double2*)A, n, nn, dpiv, n, dinfo, batch, nullptr);
    if (st == SCW_OK)
        st = scw::zgetrs(ctx->stream, (const double2*)A, n, nn, dpiv, n, (double2*)B, nrhs, (long long)n * nrhs, batch);
    ctx->launches += 3;
    std::vector<int> info(batch, 0);
    if (st == SCW_OK) {
        cudaError_t e = cudaMemcpyAsync(info.data(), dinfo, sizeof(int) * batch, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) st = fail(SCW_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaFree(dpiv);
    cudaFree(dinfo);
    if (st != SCW_OK) return st;
    int bad = 0;
    for (int b = 0; b < batch; b++) {
        if (info_host) info_host[b] = info[b];
        if (info[b]) bad = 1;
    }
    return bad ? fail(SCW_ERR_NUMERIC, "scw_zgesv: singular matrix") : SCW_OK;
}

scw_status scw_zgeev(scw_ctx ctx, int n, void* A, void* W, void* V, int batch, int* status_host) {
    if (!ctx || !A || !W || !V || n < 1 || batch < 1) return fail(SCW_ERR_ARG, "scw_zgeev: bad arguments");
    SCW_ON_DEVICE(ctx->device);
    double2* work = nullptr;
    int* dst = nullptr;
    const size_t wbytes = sizeof(double2) * ((size_t)n * n + 3 * (size_t)n) * batch;
    if (cudaMalloc(&work, wbytes) != cudaSuccess || cudaMalloc(&dst, sizeof(int) * batch) != cudaSuccess) {
        cudaFree(work);
        return fail(SCW_ERR_NOMEM, "scw_zgeev: workspace");
    }
    scw_status st = scw::zgeev(ctx->stream, (double2*)A, (double2*)W, (double2*)V, n, batch, work, dst, true);
    ctx->launches += 4;
    std::vector<int> status(batch, 0);
    if (st == SCW_OK) {
        cudaError_t e = cudaMemcpyAsync(status.data(), dst, sizeof(int) * batch, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) st = fail(SCW_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaFree(work);
    cudaFree(dst);
    if (st != SCW_OK) return st;
    int bad = 0;
    for (int b = 0; b < batch; b++) {
        if (status_host) status_host[b] = status[b];
        if (status[b]) bad = 1;
    }
    return bad ? fail(SCW_ERR_NUMERIC, "scw_zgeev: QR iteration did not converge") : SCW_OK;
}

scw_status scw_cgeev(scw_ctx ctx, int n, void* A, void* W, void* V, int batch, int* status_host) {
    if (!ctx || !A || !W || !V || n < 1 || batch < 1) return fail(SCW_ERR_ARG, "scw_cgeev: bad arguments");
    SCW_ON_DEVICE(ctx->device);
    float2* work = nullptr;
    int* dst = nullptr;
    const size_t wbytes = sizeof(float2) * ((size_t)n * n + 3 * (size_t)n) * batch;
    if (cudaMalloc(&work, wbytes) != cudaSuccess || cudaMalloc(&dst, sizeof(int) * batch) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(work);
        return fail(SCW_ERR_NOMEM, "scw_cgeev: workspace");
    }
    scw_status st = scw::geev<float2>(ctx->stream, (float2*)A, (float2*)W, (float2*)V, n, batch, work, dst, nullptr,
                                      true);
    ctx->launches += 5;
    std::vector<int> status(batch, 0);
    if (st == SCW_OK) {
        cudaError_t e = cudaMemcpyAsync(status.data(), dst, sizeof(int) * batch, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) st = fail(SCW_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaFree(work);
    cudaFree(dst);
    if (st != SCW_OK) return st;
    int bad = 0;
    for (int b = 0; b < batch; b++) {
        if (status_host) status_host[b] = status[b];
        if (status[b]) bad = 1;
    }
    return bad ? fail(SCW_ERR_NUMERIC, "scw_cgeev: QR iteration did not converge") : SCW_OK;
}

scw_status scw_set_qr_cluster(int ctas) {
    if (ctas < 0 || ctas > 8) return fail(SCW_ERR_ARG, "scw_set_qr_cluster: 0 (per call), 1 or 2..8 CTAs");
    scw::g_qr_cluster.store(ctas);
    return SCW_OK;
}

}  // extern "C"
