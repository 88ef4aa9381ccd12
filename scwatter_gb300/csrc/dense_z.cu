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
#include <cmath>
#include <vector>

#include "scw_dense.h"

namespace scw {
namespace z {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {   // conj(a) * b
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c) {   // a * b + c
    return make_double2(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
__device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ double cabs1(double2 a) { return fabs(a.x) + fabs(a.y); }
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    // Smith's algorithm
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, d = b.x + b.y * r;
        return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    }
    const double r = b.x / b.y, d = b.x * r + b.y;
    return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}

// ------------------------------------------------------------------------------------
// GEMM: C = alpha * op(A) * B + beta * C, op = identity.  64 x 64 tiles, 256 threads, each
// thread a 4 x 4 complex block; K staged 16 at a time through shared memory.
// ------------------------------------------------------------------------------------
constexpr int kGT = 64, kGK = 16;

__global__ void __launch_bounds__(256)
zgemm_kernel(int M, int N, int K, double2 alpha, const double2* __restrict__ A, int lda, long long sA,
             const double2* __restrict__ B, int ldb, long long sB, double2 beta, double2* __restrict__ C, int ldc,
             long long sC) {
    __shared__ double2 As[kGK][kGT + 1];
    __shared__ double2 Bs[kGK][kGT + 1];
    A += sA * blockIdx.z;
    B += sB * blockIdx.z;
    C += sC * blockIdx.z;
    const int i0 = blockIdx.y * kGT, j0 = blockIdx.x * kGT;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    double2 acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = make_double2(0.0, 0.0);
    for (int k0 = 0; k0 < K; k0 += kGK) {
        for (int e = threadIdx.x; e < kGK * kGT; e += 256) {
            const int r = e / kGK, kk = e % kGK;         // A tile: rows i0 + r, cols k0 + kk
            const int gi = i0 + r, gk = k0 + kk;
            As[kk][r] = (gi < M && gk < K) ? A[(long long)gi * lda + gk] : make_double2(0.0, 0.0);
            const int kk2 = e / kGT, c = e % kGT;         // B tile: rows k0 + kk2, cols j0 + c
            const int gk2 = k0 + kk2, gj = j0 + c;
            Bs[kk2][c] = (gk2 < K && gj < N) ? B[(long long)gk2 * ldb + gj] : make_double2(0.0, 0.0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kGK; kk++) {
            double2 a[4], b[4];
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
            double2* c = C + (long long)gi * ldc + gj;
            double2 v = cmul(alpha, acc[p][q]);
            if (beta.x != 0.0 || beta.y != 0.0) v = cfma(beta, *c, v);
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

__global__ void __launch_bounds__(512)
lu_panel_kernel(double2* __restrict__ A, int n, int lda, long long sA, int k0, int nb, int* __restrict__ piv,
                long long sP, int* __restrict__ info) {
    A += sA * blockIdx.x;
    piv += sP * blockIdx.x;
    __shared__ double red_v[512];
    __shared__ int red_i[512];
    __shared__ double2 pivrow[kNB];
    for (int k = k0; k < k0 + nb; k++) {
        // pivot search over rows k..n-1 of column k
        double best = -1.0;
        int bi = k;
        for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
            const double v = cabs1(A[(long long)i * lda + k]);
            if (v > best) {
                best = v;
                bi = i;
            }
        }
        red_v[threadIdx.x] = best;
        red_i[threadIdx.x] = bi;
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) {
                const double o = red_v[threadIdx.x + s];
                const int oi = red_i[threadIdx.x + s];
                if (o > red_v[threadIdx.x] || (o == red_v[threadIdx.x] && oi < red_i[threadIdx.x])) {
                    red_v[threadIdx.x] = o;
                    red_i[threadIdx.x] = oi;
                }
            }
            __syncthreads();
        }
        const int p = red_i[0];
        const bool zero = red_v[0] == 0.0;
        if (threadIdx.x == 0) {
            piv[k] = p;
            if (zero && info[blockIdx.x] == 0) info[blockIdx.x] = k + 1;
        }
        // swap rows k and p inside the panel columns k0 .. k0+nb-1
        if (p != k) {
            for (int j = k0 + threadIdx.x; j < k0 + nb; j += blockDim.x) {
                const double2 t = A[(long long)k * lda + j];
                A[(long long)k * lda + j] = A[(long long)p * lda + j];
                A[(long long)p * lda + j] = t;
            }
        }
        __syncthreads();
        const double2 d = A[(long long)k * lda + k];
        for (int j = k + 1 + threadIdx.x; j < k0 + nb; j += blockDim.x) pivrow[j - k0] = A[(long long)k * lda + j];
        __syncthreads();
        // scale the column below the pivot and update the remaining panel columns
        const double2 inv = zero ? make_double2(0.0, 0.0) : cdiv(make_double2(1.0, 0.0), d);
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) {
            double2* row = A + (long long)i * lda;
            const double2 l = cmul(row[k], inv);
            row[k] = l;
            for (int j = k + 1; j < k0 + nb; j++) row[j] = csub(row[j], cmul(l, pivrow[j - k0]));
        }
        __syncthreads();
    }
}

// apply the panel's swaps to the columns outside the panel, then solve L11 U12 = A12
__global__ void __launch_bounds__(256)
lu_swap_trsm_kernel(double2* __restrict__ A, int n, int lda, long long sA, int k0, int nb,
                    const int* __restrict__ piv, long long sP) {
    A += sA * blockIdx.y;
    piv += sP * blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;    // one column per thread
    if (j >= n || (j >= k0 && j < k0 + nb)) return;
    for (int k = k0; k < k0 + nb; k++) {
        const int p = piv[k];
        if (p != k) {
            const double2 t = A[(long long)k * lda + j];
            A[(long long)k * lda + j] = A[(long long)p * lda + j];
            A[(long long)p * lda + j] = t;
        }
    }
    if (j < k0 + nb) return;                                // columns left of the panel: swaps only
    for (int k = k0; k < k0 + nb; k++) {                    // unit lower triangular solve
        double2 v = A[(long long)k * lda + j];
        for (int m = k0; m < k; m++) v = csub(v, cmul(A[(long long)k * lda + m], A[(long long)m * lda + j]));
        A[(long long)k * lda + j] = v;
    }
}

// Row interchanges of B from zgetrf's pivots (LAPACK laswp order), one thread per column.
__global__ void __launch_bounds__(256)
laswp_kernel(const int* __restrict__ piv, long long sP, double2* __restrict__ B, int ldb, long long sB, int n,
             int nrhs) {
    piv += sP * blockIdx.y;
    B += sB * blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nrhs) return;
    for (int k = 0; k < n; k++) {
        const int p = piv[k];
        if (p != k) {
            const double2 t = B[(long long)k * ldb + j];
            B[(long long)k * ldb + j] = B[(long long)p * ldb + j];
            B[(long long)p * ldb + j] = t;
        }
    }
}

// Triangular solve restricted to the diagonal block rows [k0, k0 + nb) of the LU factors, one
// thread per right-hand-side column: unit lower L (upper == 0) or U (upper == 1).  Rows
// outside the block were already folded in by the GEMM updates of the blocked solve.
__global__ void __launch_bounds__(256)
trsm_block_kernel(const double2* __restrict__ LU, int lda, long long sA, int k0, int nb, double2* __restrict__ B,
                  int ldb, long long sB, int nrhs, int upper) {
    LU += sA * blockIdx.y;
    B += sB * blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nrhs) return;
    if (!upper) {
        for (int i = k0; i < k0 + nb; i++) {
            double2 v = B[(long long)i * ldb + j];
            const double2* row = LU + (long long)i * lda;
            for (int m = k0; m < i; m++) v = csub(v, cmul(row[m], B[(long long)m * ldb + j]));
            B[(long long)i * ldb + j] = v;
        }
    } else {
        for (int i = k0 + nb - 1; i >= k0; i--) {
            double2 v = B[(long long)i * ldb + j];
            const double2* row = LU + (long long)i * lda;
            for (int m = i + 1; m < k0 + nb; m++) v = csub(v, cmul(row[m], B[(long long)m * ldb + j]));
            B[(long long)i * ldb + j] = cdiv(v, row[i]);
        }
    }
}

// ------------------------------------------------------------------------------------
// Hessenberg reduction A -> Q^H A Q (zgehd2 semantics: H(k) = I - tau v v^H, v(k+1) = 1),
// one CTA per matrix, with the explicit unitary Q accumulated (Q := Q H(k)).
// ------------------------------------------------------------------------------------
__device__ double block_sum(double v, double* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sh[i];
    return s;
}

__global__ void __launch_bounds__(1024)
hessenberg_kernel(double2* __restrict__ A, double2* __restrict__ Q, int n, long long sA, double2* __restrict__ work) {
    A += sA * blockIdx.x;
    Q += sA * blockIdx.x;
    double2* v = work + (long long)blockIdx.x * 3 * n;      // Householder vector (rows k+1..n-1)
    double2* w = v + n;                                       // v^H A (row vector) / A v (column)
    double2* y = w + n;
    __shared__ double sh[32];
    __shared__ double2 s_tau, s_beta;
    for (int i = threadIdx.x; i < n * n; i += blockDim.x) Q[i] = make_double2((i / n) == (i % n) ? 1.0 : 0.0, 0.0);
    __syncthreads();
    for (int k = 0; k + 2 < n; k++) {
        // Householder for x = A[k+1:n, k] (zlarfg)
        double xn2 = 0.0;
        for (int i = k + 2 + threadIdx.x; i < n; i += blockDim.x) xn2 += cabs2(A[(long long)i * n + k]);
        xn2 = block_sum(xn2, sh);
        const double2 alpha = A[(long long)(k + 1) * n + k];
        if (threadIdx.x == 0) {
            if (xn2 == 0.0 && alpha.y == 0.0) {
                s_tau = make_double2(0.0, 0.0);
                s_beta = alpha;
            } else {
                const double beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
                s_tau = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
                s_beta = make_double2(beta, 0.0);
            }
        }
        __syncthreads();
        const double2 tau = s_tau;
        if (tau.x == 0.0 && tau.y == 0.0) {
            __syncthreads();
            continue;
        }
        const double2 scal = cdiv(make_double2(1.0, 0.0), csub(alpha, s_beta));
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x)
            v[i] = (i == k + 1) ? make_double2(1.0, 0.0) : cmul(A[(long long)i * n + k], scal);
        __syncthreads();
        // right: A[:, k+1:] -= tau (A[:, k+1:] v) v^H   (all rows)
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            double2 s = make_double2(0.0, 0.0);
            const double2* row = A + (long long)i * n;
            for (int j = k + 1; j < n; j++) s = cfma(row[j], v[j], s);
            y[i] = cmul(tau, s);
        }
        __syncthreads();
        for (int j = k + 1 + threadIdx.x; j < n; j += blockDim.x) {
            const double2 vc = make_double2(v[j].x, -v[j].y);
            for (int i = 0; i < n; i++) A[(long long)i * n + j] = csub(A[(long long)i * n + j], cmul(y[i], vc));
        }
        __syncthreads();
        // left: A[k+1:, k+1:] -= conj(tau) v (v^H A[k+1:, k+1:])
        for (int j = k + 1 + threadIdx.x; j < n; j += blockDim.x) {
            double2 s = make_double2(0.0, 0.0);
            for (int i = k + 1; i < n; i++) s = cfma(make_double2(v[i].x, -v[i].y), A[(long long)i * n + j], s);
            w[j] = cmul(make_double2(tau.x, -tau.y), s);
        }
        __syncthreads();
        for (int j = k + 1 + threadIdx.x; j < n; j += blockDim.x) {
            const double2 wj = w[j];
            for (int i = k + 1; i < n; i++) A[(long long)i * n + j] = csub(A[(long long)i * n + j], cmul(v[i], wj));
        }
        // column k below the subdiagonal
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x)
            A[(long long)i * n + k] = (i == k + 1) ? s_beta : make_double2(0.0, 0.0);
        // Q[:, k+1:] -= (Q[:, k+1:] v) tau v^H
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            double2 s = make_double2(0.0, 0.0);
            const double2* row = Q + (long long)i * n;
            for (int j = k + 1; j < n; j++) s = cfma(row[j], v[j], s);
            y[i] = cmul(tau, s);
        }
        __syncthreads();
        for (int j = k + 1 + threadIdx.x; j < n; j += blockDim.x) {
            const double2 vc = make_double2(v[j].x, -v[j].y);
            for (int i = 0; i < n; i++) Q[(long long)i * n + j] = csub(Q[(long long)i * n + j], cmul(y[i], vc));
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------
// Single-shift complex QR (zlahqr semantics: wantt, wantz) on the upper Hessenberg H with
// Schur vectors accumulated into Z (Z := Z G^H).  One CTA per matrix.  status[b]: 0 ok,
// 1 no convergence within 30 n iterations.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void zlartg(double2 f, double2 g, double& c, double2& s, double2& r) {
    // c s: [c, s; -conj(s), c] [f; g] = [r; 0], c real
    const double gf = cabs2(g);
    if (gf == 0.0) {
        c = 1.0;
        s = make_double2(0.0, 0.0);
        r = f;
        return;
    }
    const double ff = cabs2(f);
    if (ff == 0.0) {
        c = 0.0;
        const double ag = sqrt(gf);
        s = make_double2(g.x / ag, -g.y / ag);            // conj(g) / |g|
        r = make_double2(ag, 0.0);
        return;
    }
    const double af = sqrt(ff), d = sqrt(ff + gf);
    c = af / d;
    const double2 fs = make_double2(f.x / af, f.y / af);  // f / |f|
    s = cmulc(g, fs);                                       // conj(g) f / |f|  ... scaled below
    s = make_double2(s.x / d, s.y / d);
    r = make_double2(fs.x * d, fs.y * d);
}

__global__ void __launch_bounds__(1024)
hqr_kernel(double2* __restrict__ H, double2* __restrict__ Z, int n, long long sA, double2* __restrict__ eig,
           int* __restrict__ status) {
    H += sA * blockIdx.x;
    Z += sA * blockIdx.x;
    eig += (long long)n * blockIdx.x;
    __shared__ double s_c;
    __shared__ double2 s_s;
    __shared__ int s_l, s_done;
    const double ulp = 2.220446049250313e-16;
    const double smlnum = 2.2250738585072014e-308 * ((double)n / ulp);
    int ihi = n - 1;
    int its = 0;
    const int itmax = 30 * max(10, n);
    int total = 0;
    while (ihi >= 0) {
        // look for a small subdiagonal element in [0, ihi]
        if (threadIdx.x == 0) {
            int l = 0;
            for (int k = ihi; k > 0; k--) {
                const double2 hkk1 = H[(long long)k * n + k - 1];
                if (cabs1(hkk1) <= smlnum) {
                    l = k;
                    break;
                }
                double tst = cabs1(H[(long long)(k - 1) * n + k - 1]) + cabs1(H[(long long)k * n + k]);
                if (tst == 0.0) {
                    if (k - 2 >= 0) tst += fabs(H[(long long)(k - 1) * n + k - 2].x);
                    if (k + 1 <= ihi) tst += fabs(H[(long long)(k + 1) * n + k].x);
                }
                if (fabs(hkk1.x) <= ulp * tst) {
                    // Ahues & Tisseur conservative deflation criterion (as in zlahqr)
                    const double2 hk1k = H[(long long)(k - 1) * n + k];
                    const double2 hkk = H[(long long)k * n + k];
                    const double2 hk1k1 = H[(long long)(k - 1) * n + k - 1];
                    const double ab = fmax(cabs1(hkk1), cabs1(hk1k));
                    const double ba = fmin(cabs1(hkk1), cabs1(hk1k));
                    const double2 dd = csub(hk1k1, hkk);
                    const double aa = fmax(cabs1(hkk), cabs1(dd));
                    const double bb = fmin(cabs1(hkk), cabs1(dd));
                    const double s = aa + ab;
                    if (ba * (ab / s) <= fmax(smlnum, ulp * (bb * (aa / s)))) {
                        l = k;
                        break;
                    }
                    // coincident diagonal entries (bb = 0 above): zeroing the subdiagonal moves
                    // the two eigenvalues by at most sqrt(|h(k,k-1) h(k-1,k)|), below rounding
                    // of h(k,k) when this holds (a diagonal matrix with repeated eigenvalues
                    // and rounding-level couplings would otherwise never deflate)
                    if (ba * ab <= (ulp * cabs1(hkk)) * (ulp * cabs1(hkk))) {
                        l = k;
                        break;
                    }
                }
            }
            s_l = l;
        }
        __syncthreads();
        const int l = s_l;
        if (l > 0) {
            if (threadIdx.x == 0) H[(long long)l * n + l - 1] = make_double2(0.0, 0.0);
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
        // exceptional shifts every 10 iterations without a deflation (zlahqr's KEXSH rule)
        // shift
        if (threadIdx.x == 0) {
            double2 t;
            const double2 hii = H[(long long)ihi * n + ihi];
            if (its % 20 == 0) {
                t = make_double2(0.75 * fabs(H[(long long)ihi * n + ihi - 1].x) + hii.x, hii.y);
            } else if (its % 10 == 0) {
                t = make_double2(0.75 * fabs(H[(long long)(l + 1) * n + l].x) + H[(long long)l * n + l].x,
                                 H[(long long)l * n + l].y);
            } else {
                // Wilkinson shift from the trailing 2x2 block
                const double2 a = H[(long long)(ihi - 1) * n + ihi - 1];
                const double2 b = H[(long long)(ihi - 1) * n + ihi];
                const double2 c = H[(long long)ihi * n + ihi - 1];
                const double2 d = hii;
                const double2 half = make_double2(0.5 * (a.x - d.x), 0.5 * (a.y - d.y));
                const double2 bc = cmul(b, c);
                const double2 disc = cfma(half, half, bc);
                // complex sqrt
                const double2 sq = zsqrt(disc);
                // choose the root that makes the shift closer to d
                double2 e1 = cadd(half, sq), e2 = csub(half, sq);
                const double2 den = cabs2(e1) >= cabs2(e2) ? e1 : e2;
                t = (cabs2(den) == 0.0) ? d : csub(d, cdiv(bc, den));
            }
            s_s = t;                                      // reuse as shift storage
        }
        __syncthreads();
        const double2 shift = s_s;
        __syncthreads();
        // implicit single-shift QR sweep over the active block [l, ihi]
        for (int k = l; k < ihi; k++) {
            if (threadIdx.x == 0) {
                double2 f, g;
                if (k == l) {
                    f = csub(H[(long long)l * n + l], shift);
                    g = H[(long long)(l + 1) * n + l];
                } else {
                    f = H[(long long)k * n + k - 1];
                    g = H[(long long)(k + 1) * n + k - 1];
                }
                double c;
                double2 s, r;
                zlartg(f, g, c, s, r);
                if (k > l) {
                    H[(long long)k * n + k - 1] = r;
                    H[(long long)(k + 1) * n + k - 1] = make_double2(0.0, 0.0);
                }
                s_c = c;
                s_s = s;
            }
            __syncthreads();
            const double c = s_c;
            const double2 s = s_s;
            // rows k, k+1, columns from k (or k-1 handled above) to n-1:  G [x; y]
            for (int j = k + threadIdx.x; j < n; j += blockDim.x) {
                const double2 x = H[(long long)k * n + j], yv = H[(long long)(k + 1) * n + j];
                H[(long long)k * n + j] = make_double2(c * x.x + (s.x * yv.x - s.y * yv.y), c * x.y + (s.x * yv.y + s.y * yv.x));
                // -conj(s) x + c y
                H[(long long)(k + 1) * n + j] = make_double2(c * yv.x - (s.x * x.x + s.y * x.y), c * yv.y - (s.x * x.y - s.y * x.x));
            }
            __syncthreads();
            // columns k, k+1, rows 0 .. min(k+2, ihi):  [x, y] G^H
            const int rmax = min(k + 2, ihi);
            for (int i = threadIdx.x; i <= rmax; i += blockDim.x) {
                const double2 x = H[(long long)i * n + k], yv = H[(long long)i * n + k + 1];
                // x c + y conj(s);  -x s + y c
                H[(long long)i * n + k] = make_double2(c * x.x + (yv.x * s.x + yv.y * s.y), c * x.y + (yv.y * s.x - yv.x * s.y));
                H[(long long)i * n + k + 1] = make_double2(c * yv.x - (x.x * s.x - x.y * s.y), c * yv.y - (x.x * s.y + x.y * s.x));
            }
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const double2 x = Z[(long long)i * n + k], yv = Z[(long long)i * n + k + 1];
                Z[(long long)i * n + k] = make_double2(c * x.x + (yv.x * s.x + yv.y * s.y), c * x.y + (yv.y * s.x - yv.x * s.y));
                Z[(long long)i * n + k + 1] = make_double2(c * yv.x - (x.x * s.x - x.y * s.y), c * yv.y - (x.x * s.y + x.y * s.x));
            }
            __syncthreads();
        }
    }
    (void)s_done;
}

// ------------------------------------------------------------------------------------
// Eigenvectors of the upper triangular Schur factor T (ztrevc semantics, right vectors):
// X[:, k] solves (T - T_kk I) x = 0 with x_k = 1, x_i = 0 for i > k.  One warp per vector.
// X is written row-major (column k = eigenvector k).
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
trevc_kernel(const double2* __restrict__ T, double2* __restrict__ X, int n, long long sA) {
    T += sA * blockIdx.y;
    X += sA * blockIdx.y;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n) return;
    const int k = warp;
    const double ulp = 2.220446049250313e-16;
    const double2 lam = T[(long long)k * n + k];
    const double smin = fmax(ulp * cabs1(lam), 2.2250738585072014e-308 * ((double)n / ulp));
    // x_k = 1, x_{k+1..} = 0
    for (int i = lane; i < n; i += 32) X[(long long)i * n + k] = make_double2(i == k ? 1.0 : 0.0, 0.0);
    __syncwarp();
    for (int i = k - 1; i >= 0; i--) {
        // x_i = -(sum_{j=i+1..k} T_ij x_j) / (T_ii - lam)
        double2 s = make_double2(0.0, 0.0);
        for (int j = i + 1 + lane; j <= k; j += 32) s = cfma(T[(long long)i * n + j], X[(long long)j * n + k], s);
        for (int o = 16; o > 0; o >>= 1) {
            s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
            s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
        }
        if (lane == 0) {
            double2 d = csub(T[(long long)i * n + i], lam);
            if (cabs1(d) < smin) d = make_double2(smin, 0.0);
            X[(long long)i * n + k] = cdiv(make_double2(-s.x, -s.y), d);
        }
        __syncwarp();
    }
}

}  // namespace z

// ------------------------------------------------------------------------------------
// Host wrappers
// ------------------------------------------------------------------------------------
scw_status zgemm(cudaStream_t st, int M, int N, int K, double2 alpha, const double2* A, int lda, long long sA,
                 const double2* B, int ldb, long long sB, double2 beta, double2* C, int ldc, long long sC,
                 int batch) {
    if (M <= 0 || N <= 0 || batch <= 0) return SCW_OK;
    dim3 grid((N + z::kGT - 1) / z::kGT, (M + z::kGT - 1) / z::kGT, batch);
    z::zgemm_kernel<<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC);
    SCW_CUDA_TRY(cudaGetLastError());
    return SCW_OK;
}

scw_status zgetrf(cudaStream_t st, double2* A, int n, long long sA, int* piv, long long sP, int* info, int batch,
                  double2* /*unused*/) {
    if (n <= 0 || batch <= 0) return SCW_OK;
    SCW_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(int) * batch, st));
    for (int k0 = 0; k0 < n; k0 += z::kNB) {
        const int nb = std::min(z::kNB, n - k0);
        z::lu_panel_kernel<<<batch, 512, 0, st>>>(A, n, n, sA, k0, nb, piv, sP, info);
        SCW_CUDA_TRY(cudaGetLastError());
        dim3 g2((n + 255) / 256, batch);
        z::lu_swap_trsm_kernel<<<g2, 256, 0, st>>>(A, n, n, sA, k0, nb, piv, sP);
        SCW_CUDA_TRY(cudaGetLastError());
        const int rem = n - k0 - nb;
        if (rem > 0) {
            // A22 -= L21 U12
            scw_status s = zgemm(st, rem, rem, nb, make_double2(-1.0, 0.0), A + (long long)(k0 + nb) * n + k0, n, sA,
                                 A + (long long)k0 * n + k0 + nb, n, sA, make_double2(1.0, 0.0),
                                 A + (long long)(k0 + nb) * n + k0 + nb, n, sA, batch);
            if (s != SCW_OK) return s;
        }
    }
    return SCW_OK;
}

scw_status zgetrs(cudaStream_t st, const double2* LU, int n, long long sA, const int* piv, long long sP, double2* B,
                  int nrhs, long long sB, int batch) {
    // blocked: per diagonal block a small triangular solve, the rest of the rows updated by GEMM
    if (n <= 0 || nrhs <= 0 || batch <= 0) return SCW_OK;
    constexpr int kTB = 64;
    const dim3 g((nrhs + 255) / 256, batch);
    z::laswp_kernel<<<g, 256, 0, st>>>(piv, sP, B, nrhs, sB, n, nrhs);
    SCW_CUDA_TRY(cudaGetLastError());
    for (int k0 = 0; k0 < n; k0 += kTB) {
        const int nb = std::min(kTB, n - k0);
        z::trsm_block_kernel<<<g, 256, 0, st>>>(LU, n, sA, k0, nb, B, nrhs, sB, nrhs, 0);
        SCW_CUDA_TRY(cudaGetLastError());
        const int rem = n - k0 - nb;
        if (rem > 0) {
            scw_status s = zgemm(st, rem, nrhs, nb, make_double2(-1.0, 0.0), LU + (long long)(k0 + nb) * n + k0, n, sA,
                                 B + (long long)k0 * nrhs, nrhs, sB, make_double2(1.0, 0.0),
                                 B + (long long)(k0 + nb) * nrhs, nrhs, sB, batch);
            if (s != SCW_OK) return s;
        }
    }
    for (int k0 = ((n - 1) / kTB) * kTB; k0 >= 0; k0 -= kTB) {
        const int nb = std::min(kTB, n - k0);
        z::trsm_block_kernel<<<g, 256, 0, st>>>(LU, n, sA, k0, nb, B, nrhs, sB, nrhs, 1);
        SCW_CUDA_TRY(cudaGetLastError());
        if (k0 > 0) {
            scw_status s = zgemm(st, k0, nrhs, nb, make_double2(-1.0, 0.0), LU + k0, n, sA, B + (long long)k0 * nrhs,
                                 nrhs, sB, make_double2(1.0, 0.0), B, nrhs, sB, batch);
            if (s != SCW_OK) return s;
        }
    }
    return SCW_OK;
}

scw_status zgehrd(cudaStream_t st, double2* A, double2* Q, int n, int batch, double2* work) {
    if (n <= 0 || batch <= 0) return SCW_OK;
    z::hessenberg_kernel<<<batch, 1024, 0, st>>>(A, Q, n, (long long)n * n, work);
    SCW_CUDA_TRY(cudaGetLastError());
    return SCW_OK;
}

scw_status zgeev(cudaStream_t st, double2* A, double2* W, double2* V, int n, int batch, double2* work, int* status) {
    // A (overwritten): n x n per batch entry; W: n eigenvalues; V: n x n right eigenvectors (columns)
    // work: >= batch * (n*n + 3 n) double2
    if (n <= 0 || batch <= 0) return SCW_OK;
    const long long nn = (long long)n * n;
    double2* Q = work;                       // batch * n * n: Schur vectors
    double2* hw = work + nn * batch;         // batch * 3n
    SCW_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int) * batch, st));
    z::hessenberg_kernel<<<batch, 1024, 0, st>>>(A, Q, n, nn, hw);
    SCW_CUDA_TRY(cudaGetLastError());
    z::hqr_kernel<<<batch, 1024, 0, st>>>(A, Q, n, nn, W, status);
    SCW_CUDA_TRY(cudaGetLastError());
    // X (triangular eigenvectors) into V, then V := Q X
    dim3 gt((n * 32 + 255) / 256, batch);
    z::trevc_kernel<<<gt, 256, 0, st>>>(A, V, n, nn);
    SCW_CUDA_TRY(cudaGetLastError());
    // A is free now: A := Q X, then copy to V
    scw_status s = zgemm(st, n, n, n, make_double2(1.0, 0.0), Q, n, nn, V, n, nn, make_double2(0.0, 0.0), A, n, nn, batch);
    if (s != SCW_OK) return s;
    SCW_CUDA_TRY(cudaMemcpyAsync(V, A, sizeof(double2) * nn * batch, cudaMemcpyDeviceToDevice, st));
    return SCW_OK;
}

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
    SCW_CUDA_TRY(cudaSetDevice(ctx->device));
    ctx->launches++;
    return scw::zgemm(ctx->stream, M, N, K, make_double2(alpha[0], alpha[1]), (const double2*)A, K, (long long)M * K,
                      (const double2*)B, N, (long long)K * N, make_double2(beta[0], beta[1]), (double2*)C, N,
                      (long long)M * N, batch);
}

scw_status scw_zgesv(scw_ctx ctx, int n, int nrhs, void* A, void* B, int batch, int* info_host) {
    if (!ctx || !A || !B || n < 1 || nrhs < 1 || batch < 1) return fail(SCW_ERR_ARG, "scw_zgesv: bad arguments");
    SCW_CUDA_TRY(cudaSetDevice(ctx->device));
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
    SCW_CUDA_TRY(cudaSetDevice(ctx->device));
    double2* work = nullptr;
    int* dst = nullptr;
    const size_t wbytes = sizeof(double2) * ((size_t)n * n + 3 * (size_t)n) * batch;
    if (cudaMalloc(&work, wbytes) != cudaSuccess || cudaMalloc(&dst, sizeof(int) * batch) != cudaSuccess) {
        cudaFree(work);
        return fail(SCW_ERR_NOMEM, "scw_zgeev: workspace");
    }
    scw_status st = scw::zgeev(ctx->stream, (double2*)A, (double2*)W, (double2*)V, n, batch, work, dst);
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

}  // extern "C"
