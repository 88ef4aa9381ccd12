// Mixed-precision eigen-solver of the reduced layer matrices.  The reference eigendecomposes
// every layer matrix with LAPACKE_zgeev in FP64 (third_Lapack.h:38-47, called from
// sCWatter.cpp:248-272).  Here the Householder + QR factorisation runs in FP32 (the GB300 FP32
// rate is 64x its FP64 rate), and Newton refinement of all eigenpairs at once restores FP64
// accuracy.  A slice that does not reach the residual tolerance goes through the FP64
// Householder + QR solver, so every accepted result is FP64-accurate by its residual.
// The algorithm is in scw_eigmix.h.
#include <algorithm>
#include <cmath>

#include "scw_complex.cuh"
#include "scw_dense.h"
#include "scw_eigmix.h"

namespace scw {
namespace mx {

using z::CT;
using z::cabs1;
using z::cabs2;
using z::cdiv;
using z::cfma;
using z::cmul;
using z::csub;

static unsigned nblk(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

#define MX_TRY(expr)                           \
    do {                                       \
        scw_status s_ = (expr);                \
        if (s_ != SCW_OK) return s_;           \
    } while (0)
#define MX_LAUNCHED(count)                     \
    do {                                       \
        SCW_CUDA_TRY(cudaGetLastError());      \
        if (launches) *launches += (count);    \
    } while (0)

size_t eigmix_small_bytes(int n, int Z) {
    EigMixWs w{};
    eigmix_carve_small(w, nullptr, n, Z);
    return (size_t)reinterpret_cast<uintptr_t>(w.res) + sizeof(double) * Z + 256;
}

void eigmix_carve_small(EigMixWs& w, char* base, int n, int Z) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        off = (off + 255) / 256 * 256;
        char* p = base + off;
        off += std::max<size_t>(bytes, 1);
        return p;
    };
    const size_t zn = (size_t)Z * n;
    w.label = (int*)take(sizeof(int) * zn);
    w.member = (int*)take(sizeof(int) * zn);
    w.cstart = (int*)take(sizeof(int) * (size_t)Z * (n + 1));
    w.ncl = (int*)take(sizeof(int) * Z);
    w.piv = (int*)take(sizeof(int) * zn);
    w.info = (int*)take(sizeof(int) * Z);
    w.qr = (int*)take(sizeof(int) * Z);
    w.state = (int*)take(sizeof(int) * Z);
    w.steps = (int*)take(sizeof(int) * Z);
    w.Y = (double2*)take(sizeof(double2) * zn * kMaxCluster);
    w.rn = (double*)take(sizeof(double) * zn);
    w.xn = (double*)take(sizeof(double) * zn);
    w.anorm = (double*)take(sizeof(double) * Z);
    w.res = (double*)take(sizeof(double) * Z);
}

// slice states: refining, converged, or the reason it goes to the FP64 solver
enum : int {
    kRefining = 0,
    kConverged = 1,
    kQrFailed = 2,          // FP32 QR iteration did not converge
    kClusterTooLarge = 3,   // a cluster above kMaxCluster eigenvalues (or label propagation did not settle)
    kSingularX = 4,         // zero pivot in the FP32 LU of the eigenvector matrix
    kClusterFailed = 5,     // the small FP64 Schur solve of a cluster did not converge
    kNotConverged = 6       // residual above tol_accept after the last step
};

// ||A||_1 (largest column sum of |a_ij|) per matrix
__global__ void __launch_bounds__(256) norm1_kernel(const double2* __restrict__ A, int n, double* __restrict__ anorm) {
    A += (long long)n * n * blockIdx.x;
    __shared__ double red[256];
    double best = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < n; i++) {
            const double2 a = A[(long long)i * n + j];
            s += hypot(a.x, a.y);
        }
        best = fmax(best, s);
    }
    red[threadIdx.x] = best;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) anorm[blockIdx.x] = red[0];
}

__global__ void to_f32_kernel(const double2* __restrict__ A, float2* __restrict__ B, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
        B[i] = make_float2((float)A[i].x, (float)A[i].y);
}

// FP32 eigenpairs -> FP64 starting point; state from the FP32 QR status
__global__ void init_kernel(const float2* __restrict__ lam32, const float2* __restrict__ X32, double2* __restrict__ lam,
                            double2* __restrict__ X, int n, const int* __restrict__ qr, int* __restrict__ state,
                            int* __restrict__ steps, double* __restrict__ res) {
    const int b = blockIdx.y;
    const long long nn = (long long)n * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = X32[nn * b + i];
        X[nn * b + i] = make_double2(v.x, v.y);
        if (i < n) {
            const float2 l = lam32[(long long)n * b + i];
            lam[(long long)n * b + i] = make_double2(l.x, l.y);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        state[b] = qr[b] ? kQrFailed : kRefining;
        steps[b] = -1;
        res[b] = INFINITY;
    }
}

// Clusters: connected components of the graph |lambda_i - lambda_j| < tau_rel ||A||_1, by
// minimum-label propagation with pointer jumping (at most 64 passes, else the slice is
// rejected).  Components of two or more members get ids 0.. in the order of their smallest
// member; their members are listed in increasing order.  label[i] = cluster id or -1.
__global__ void __launch_bounds__(1024)
cluster_kernel(const double2* __restrict__ lam, int n, const double* __restrict__ anorm, double tau_rel,
               int* __restrict__ label, int* __restrict__ member, int* __restrict__ cstart, int* __restrict__ ncl,
               int* __restrict__ state) {
    const int b = blockIdx.x;
    extern __shared__ __align__(16) unsigned char smem[];
    double2* lm = reinterpret_cast<double2*>(smem);
    int* lab = reinterpret_cast<int*>(lm + n);
    int* cnt = lab + n;
    int* cid = cnt + n;
    int* nxt = cid + n;
    __shared__ int changed, reject;
    lam += (long long)n * b;
    label += (long long)n * b;
    member += (long long)n * b;
    cstart += (long long)(n + 1) * b;
    if (state[b] != kRefining) {
        if (threadIdx.x == 0) ncl[b] = 0;
        return;
    }
    const double tau = tau_rel * anorm[b], tau2 = tau * tau;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        lm[i] = lam[i];
        lab[i] = i;
        cnt[i] = 0;
    }
    if (threadIdx.x == 0) reject = 0;
    __syncthreads();
    int pass = 0;
    for (; pass < 64; pass++) {
        if (threadIdx.x == 0) changed = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double2 li = lm[i];
            int m = lab[i];
            for (int j = 0; j < n; j++) {
                const double dx = lm[j].x - li.x, dy = lm[j].y - li.y;
                if (dx * dx + dy * dy < tau2) m = min(m, lab[j]);
            }
            if (m < lab[i]) {
                lab[i] = m;
                changed = 1;
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) lab[i] = lab[lab[i]];
        __syncthreads();
        if (!changed) break;
        __syncthreads();
    }
    if (pass == 64) {
        if (threadIdx.x == 0) {
            state[b] = kClusterTooLarge;
            ncl[b] = 0;
        }
        return;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&cnt[lab[i]], 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        int c = 0, pos = 0;
        for (int r = 0; r < n; r++) {
            cid[r] = -1;
            if (lab[r] == r && cnt[r] > 1) {
                if (cnt[r] > kMaxCluster) reject = 1;
                cid[r] = c;
                cstart[c] = pos;
                nxt[c] = pos;
                pos += cnt[r];
                c++;
            }
        }
        cstart[c] = pos;
        ncl[b] = c;
        for (int i = 0; i < n; i++) {
            const int id = cid[lab[i]];
            label[i] = id;
            if (id >= 0) member[nxt[id]++] = i;
        }
        if (reject) {
            state[b] = kClusterTooLarge;
            ncl[b] = 0;
        }
    }
}

// R = (A X) - X diag(lambda) from the FP64 product AX: R rounded to FP32 (the right-hand side
// of E = X^-1 R) and the column sums of |r_ij|^2 and |x_ij|^2.  Block: 32 columns x 8 row lanes.
__global__ void __launch_bounds__(256)
resid_kernel(const double2* __restrict__ AX, const double2* __restrict__ X, const double2* __restrict__ lam, int n,
             float2* __restrict__ R32, double* __restrict__ rn, double* __restrict__ xn, const int* __restrict__ state) {
    const int b = blockIdx.y;
    if (state[b] != kRefining) return;
    const long long nn = (long long)n * n;
    AX += nn * b;
    X += nn * b;
    R32 += nn * b;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int j = blockIdx.x * 32 + tx;
    __shared__ double sr[8][32], sx[8][32];
    double ar = 0.0, axx = 0.0;
    if (j < n) {
        const double2 l = lam[(long long)n * b + j];
        for (int i = ty; i < n; i += 8) {
            const long long o = (long long)i * n + j;
            const double2 x = X[o];
            const double2 r = csub(AX[o], cmul(x, l));
            R32[o] = make_float2((float)r.x, (float)r.y);
            ar += cabs2(r);
            axx += cabs2(x);
        }
    }
    sr[ty][tx] = ar;
    sx[ty][tx] = axx;
    __syncthreads();
    if (ty == 0 && j < n) {
        double a = 0.0, c = 0.0;
        for (int t = 0; t < 8; t++) {
            a += sr[t][tx];
            c += sx[t][tx];
        }
        rn[(long long)n * b + j] = a;
        xn[(long long)n * b + j] = c;
    }
}

// max relative column residual; converged slices stop refining
__global__ void __launch_bounds__(256)
gate_kernel(int n, const double* __restrict__ rn, const double* __restrict__ xn, const double* __restrict__ anorm,
            double tol, int step, int* __restrict__ state, int* __restrict__ steps, double* __restrict__ res) {
    // tol: the stopping tolerance at early checks, the acceptance tolerance from step `steps` on
    const int b = blockIdx.x;
    if (state[b] != kRefining) return;
    __shared__ double red[256];
    double worst = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double x = xn[(long long)n * b + j];
        const double r = x > 0.0 ? sqrt(rn[(long long)n * b + j] / x) : INFINITY;
        worst = (r > worst || r != r) ? r : worst;
    }
    red[threadIdx.x] = worst;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            const double o = red[threadIdx.x + s];
            if (o > red[threadIdx.x] || o != o) red[threadIdx.x] = o;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double r = red[0] / anorm[b];
        res[b] = r;
        if (r <= tol) {
            state[b] = kConverged;
            steps[b] = step;
        }
    }
}

// X (FP64) rounded to FP32 twice: the LU input and the GEMM operand
__global__ void to32_kernel(const double2* __restrict__ X, float2* __restrict__ L, float2* __restrict__ X32, int n,
                            const int* __restrict__ state) {
    const int b = blockIdx.y;
    if (state[b] != kRefining) return;
    const long long nn = (long long)n * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x) {
        const double2 v = X[nn * b + i];
        const float2 f = make_float2((float)v.x, (float)v.y);
        L[nn * b + i] = f;
        X32[nn * b + i] = f;
    }
}

__global__ void lu_check_kernel(const int* __restrict__ info, int Z, int* __restrict__ state) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < Z && state[b] == kRefining && info[b] != 0) state[b] = kSingularX;
}

// lambda_i += E_ii for eigenvalues outside every cluster
__global__ void singleton_kernel(const float2* __restrict__ E, const int* __restrict__ label, double2* __restrict__ lam,
                                 int n, const int* __restrict__ state) {
    const int b = blockIdx.y;
    if (state[b] != kRefining) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || label[(long long)n * b + i] >= 0) return;
    const float2 e = E[(long long)n * n * b + (long long)i * n + i];
    double2& l = lam[(long long)n * b + i];
    l = make_double2(l.x + (double)e.x, l.y + (double)e.y);
}

// Small eigenproblem of one cluster (k <= kMaxCluster, one CTA of kMaxCluster threads):
// M = diag(lambda_S) + E_SS in FP64 -> Householder Hessenberg form -> single-shift complex QR
// (Schur form T, unitary U) -> eigenvectors of T with pairs closer than deg_rel ||A||_1 left
// uncoupled (a degenerate eigenvalue keeps the unitary Schur basis) -> Y = U Yt.
// Y goes to Yout (k x k, row-major, at the cluster's slot), the eigenvalues to lambda.
__global__ void __launch_bounds__(kMaxCluster)
cluster_eig_kernel(const float2* __restrict__ E, const int* __restrict__ member, const int* __restrict__ cstart,
                   const int* __restrict__ ncl, double2* __restrict__ lam, int n, const double* __restrict__ anorm,
                   double deg_rel, double2* __restrict__ Yout, int* __restrict__ state) {
    const int b = blockIdx.y, c = blockIdx.x;
    if (state[b] != kRefining || c >= ncl[b]) return;
    extern __shared__ __align__(16) unsigned char smem[];
    const int* cs = cstart + (long long)(n + 1) * b;
    const int s0 = cs[c], k = cs[c + 1] - s0;
    const int* mem = member + (long long)n * b + s0;
    double2* T = reinterpret_cast<double2*>(smem);
    double2* U = T + k * k;
    double2* Yt = U + k * k;
    __shared__ double2 v[kMaxCluster];
    __shared__ double red[kMaxCluster];
    __shared__ double2 s_tau, s_beta, s_s;
    __shared__ double s_c;
    __shared__ int s_l, s_fail;
    const int t = threadIdx.x;
    const long long nn = (long long)n * n;
    E += nn * b;
    lam += (long long)n * b;
    if (t < k) {
        const int mi = mem[t];
        for (int j = 0; j < k; j++) {
            const float2 e = E[(long long)mi * n + mem[j]];
            double2 m = make_double2(e.x, e.y);
            if (j == t) m = make_double2(m.x + lam[mi].x, m.y + lam[mi].y);
            T[t * k + j] = m;
            U[t * k + j] = make_double2(j == t ? 1.0 : 0.0, 0.0);
        }
    }
    if (t == 0) s_fail = 0;
    __syncthreads();
    // Householder reduction to Hessenberg form, U := U H(p)
    for (int p = 0; p + 2 < k; p++) {
        double x2 = 0.0;
        if (t >= p + 2 && t < k) x2 = cabs2(T[t * k + p]);
        red[t] = x2;
        __syncthreads();
        if (t == 0) {
            double xn2 = 0.0;
            for (int i = 0; i < kMaxCluster; i++) xn2 += red[i];
            const double2 alpha = T[(p + 1) * k + p];
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
        const double2 alpha = T[(p + 1) * k + p];
        const double2 scal = cdiv(make_double2(1.0, 0.0), csub(alpha, s_beta));
        if (t >= p + 1 && t < k) v[t] = (t == p + 1) ? make_double2(1.0, 0.0) : cmul(T[t * k + p], scal);
        __syncthreads();
        // right: row t of T[:, p+1:] -= tau (row . v) v^H
        if (t < k) {
            double2 s = make_double2(0.0, 0.0);
            for (int j = p + 1; j < k; j++) s = cfma(T[t * k + j], v[j], s);
            const double2 y = cmul(tau, s);
            for (int j = p + 1; j < k; j++) T[t * k + j] = csub(T[t * k + j], cmul(y, make_double2(v[j].x, -v[j].y)));
        }
        __syncthreads();
        // left: column t of T[p+1:, p+1:] -= conj(tau) v (v^H column)
        if (t >= p + 1 && t < k) {
            double2 s = make_double2(0.0, 0.0);
            for (int i = p + 1; i < k; i++) s = cfma(make_double2(v[i].x, -v[i].y), T[i * k + t], s);
            const double2 w = cmul(make_double2(tau.x, -tau.y), s);
            for (int i = p + 1; i < k; i++) T[i * k + t] = csub(T[i * k + t], cmul(v[i], w));
        }
        __syncthreads();
        if (t >= p + 1 && t < k) T[t * k + p] = (t == p + 1) ? s_beta : make_double2(0.0, 0.0);
        if (t < k) {
            double2 s = make_double2(0.0, 0.0);
            for (int j = p + 1; j < k; j++) s = cfma(U[t * k + j], v[j], s);
            const double2 y = cmul(tau, s);
            for (int j = p + 1; j < k; j++) U[t * k + j] = csub(U[t * k + j], cmul(y, make_double2(v[j].x, -v[j].y)));
        }
        __syncthreads();
    }
    // single-shift complex QR with Schur vectors (the rules of hqr_kernel)
    int ihi = k - 1, its = 0, total = 0;
    const int itmax = 30 * max(10, k);
    while (ihi >= 0) {
        if (t == 0) {
            int l = 0;
            for (int kk = ihi; kk > 0; kk--)
                if (z::hqr_deflates(T, k, kk, ihi)) {
                    l = kk;
                    break;
                }
            s_l = l;
            if (l > 0) T[l * k + l - 1] = make_double2(0.0, 0.0);
        }
        __syncthreads();
        const int l = s_l;
        if (l >= ihi) {
            ihi = l - 1;
            its = 0;
            __syncthreads();
            continue;
        }
        if (total > itmax) {
            if (t == 0) s_fail = 1;
            break;
        }
        its++;
        total++;
        if (t == 0) {
            double2 sh;
            const double2 hii = T[ihi * k + ihi];
            if (its % 20 == 0) {
                sh = make_double2(0.75 * fabs(T[ihi * k + ihi - 1].x) + hii.x, hii.y);
            } else if (its % 10 == 0) {
                sh = make_double2(0.75 * fabs(T[(l + 1) * k + l].x) + T[l * k + l].x, T[l * k + l].y);
            } else {
                const double2 a = T[(ihi - 1) * k + ihi - 1], bq = T[(ihi - 1) * k + ihi], cq = T[ihi * k + ihi - 1];
                const double2 half = make_double2(0.5 * (a.x - hii.x), 0.5 * (a.y - hii.y));
                const double2 bc = cmul(bq, cq);
                const double2 sq = zsqrt(cfma(half, half, bc));
                const double2 e1 = z::cadd(half, sq), e2 = csub(half, sq);
                const double2 den = cabs2(e1) >= cabs2(e2) ? e1 : e2;
                sh = (cabs2(den) == 0.0) ? hii : csub(hii, cdiv(bc, den));
            }
            s_s = sh;
        }
        __syncthreads();
        const double2 shift = s_s;
        __syncthreads();
        for (int q = l; q < ihi; q++) {
            if (t == 0) {
                double2 f, g, s, r;
                double cc;
                if (q == l) {
                    f = csub(T[l * k + l], shift);
                    g = T[(l + 1) * k + l];
                } else {
                    f = T[q * k + q - 1];
                    g = T[(q + 1) * k + q - 1];
                }
                z::zlartg(f, g, cc, s, r);
                if (q > l) {
                    T[q * k + q - 1] = r;
                    T[(q + 1) * k + q - 1] = make_double2(0.0, 0.0);
                }
                s_c = cc;
                s_s = s;
            }
            __syncthreads();
            const double cc = s_c;
            const double2 s = s_s;
            if (t >= q && t < k) {
                const double2 x = T[q * k + t], y = T[(q + 1) * k + t];
                T[q * k + t] = make_double2(cc * x.x + (s.x * y.x - s.y * y.y), cc * x.y + (s.x * y.y + s.y * y.x));
                T[(q + 1) * k + t] = make_double2(cc * y.x - (s.x * x.x + s.y * x.y), cc * y.y - (s.x * x.y - s.y * x.x));
            }
            __syncthreads();
            if (t <= min(q + 2, ihi)) {
                const double2 x = T[t * k + q], y = T[t * k + q + 1];
                T[t * k + q] = make_double2(cc * x.x + (y.x * s.x + y.y * s.y), cc * x.y + (y.y * s.x - y.x * s.y));
                T[t * k + q + 1] = make_double2(cc * y.x - (x.x * s.x - x.y * s.y), cc * y.y - (x.x * s.y + x.y * s.x));
            }
            if (t < k) {
                const double2 x = U[t * k + q], y = U[t * k + q + 1];
                U[t * k + q] = make_double2(cc * x.x + (y.x * s.x + y.y * s.y), cc * x.y + (y.y * s.x - y.x * s.y));
                U[t * k + q + 1] = make_double2(cc * y.x - (x.x * s.x - x.y * s.y), cc * y.y - (x.x * s.y + x.y * s.x));
            }
            __syncthreads();
        }
    }
    __syncthreads();
    if (s_fail) {
        if (t == 0) state[b] = kClusterFailed;
        return;
    }
    // eigenvectors of T: column t, unit diagonal, degenerate pairs uncoupled
    const double deg = deg_rel * anorm[b];
    if (t < k) {
        for (int i = 0; i < k; i++) Yt[i * k + t] = make_double2(i == t ? 1.0 : 0.0, 0.0);
        const double2 lt = T[t * k + t];
        for (int i = t - 1; i >= 0; i--) {
            double2 s = make_double2(0.0, 0.0);
            for (int m = i + 1; m <= t; m++) s = cfma(T[i * k + m], Yt[m * k + t], s);
            const double2 d = csub(T[i * k + i], lt);
            Yt[i * k + t] = (hypot(d.x, d.y) <= deg) ? make_double2(0.0, 0.0) : cdiv(make_double2(-s.x, -s.y), d);
        }
    }
    __syncthreads();
    if (t < k) {
        double2* Yc = Yout + ((long long)n * b + s0) * kMaxCluster;
        for (int i = 0; i < k; i++) {
            double2 s = make_double2(0.0, 0.0);
            for (int m = 0; m < k; m++) s = cfma(U[i * k + m], Yt[m * k + t], s);
            Yc[i * k + t] = s;
        }
        lam[mem[t]] = T[t * k + t];
    }
}

// F_ij = E_ij / (lambda_j - lambda_i) between different clusters / singletons, 0 within one
__global__ void f_kernel(const float2* __restrict__ E, const double2* __restrict__ lam, const int* __restrict__ label,
                         int n, float2* __restrict__ F, const int* __restrict__ state) {
    const int b = blockIdx.y;
    if (state[b] != kRefining) return;
    const long long nn = (long long)n * n;
    E += nn * b;
    F += nn * b;
    lam += (long long)n * b;
    label += (long long)n * b;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / n), j = (int)(e % n);
        const int li = label[i], lj = label[j];
        float2 f = make_float2(0.f, 0.f);
        if (i != j && !(li >= 0 && li == lj)) {
            const double2 d = csub(lam[j], lam[i]);
            if (d.x != 0.0 || d.y != 0.0) {
                const double2 q = cdiv(make_double2(E[e].x, E[e].y), d);
                f = make_float2((float)q.x, (float)q.y);
            }
        }
        F[e] = f;
    }
}

__global__ void xupdate_kernel(const float2* __restrict__ P, double2* __restrict__ X, int n, const int* __restrict__ state) {
    const int b = blockIdx.y;
    if (state[b] != kRefining) return;
    const long long nn = (long long)n * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x) {
        const float2 p = P[nn * b + i];
        double2& x = X[nn * b + i];
        x = make_double2(x.x + (double)p.x, x.y + (double)p.y);
    }
}

// X[:, S] := X[:, S] Y_S for every cluster S (one CTA of kMaxCluster threads per cluster; each
// thread stages its row's k entries in shared memory)
__global__ void __launch_bounds__(kMaxCluster)
rotate_kernel(double2* __restrict__ X, const int* __restrict__ member, const int* __restrict__ cstart,
              const int* __restrict__ ncl, const double2* __restrict__ Yin, int n, const int* __restrict__ state) {
    const int b = blockIdx.y, c = blockIdx.x;
    if (state[b] != kRefining || c >= ncl[b]) return;
    extern __shared__ __align__(16) unsigned char smem[];
    const int* cs = cstart + (long long)(n + 1) * b;
    const int s0 = cs[c], k = cs[c + 1] - s0;
    const int* mem = member + (long long)n * b + s0;
    double2* Ys = reinterpret_cast<double2*>(smem);
    double2* xs = Ys + k * k + threadIdx.x * k;
    const double2* Yc = Yin + ((long long)n * b + s0) * kMaxCluster;
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) Ys[e] = Yc[e];
    __syncthreads();
    X += (long long)n * n * b;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double2* row = X + (long long)i * n;
        for (int l = 0; l < k; l++) xs[l] = row[mem[l]];
        for (int j = 0; j < k; j++) {
            double2 s = make_double2(0.0, 0.0);
            for (int l = 0; l < k; l++) s = cfma(xs[l], Ys[l * k + j], s);
            row[mem[j]] = s;
        }
    }
}

__global__ void final_kernel(int* __restrict__ state, int* __restrict__ accepted, int Z) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= Z) return;
    if (state[b] == kRefining) state[b] = kNotConverged;
    accepted[b] = state[b] == kConverged;
}

static scw_status set_smem(const void* fn, size_t bytes) {
    SCW_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return SCW_OK;
}

scw_status geev_mixed(cudaStream_t st, double2* A, double2* lam, double2* V, int n, int Z, const EigMixWs& w,
                      double2* fb_work, int* status, const EigMixParams& prm, long long* launches) {
    if (n <= 0 || Z <= 0) return SCW_OK;
    if (n > kMaxN) return fail(SCW_ERR_ARG, "geev_mixed: matrix order above the mixed path's limit");
    const long long nn = (long long)n * n;
    if (w.hw != w.S1 + nn * Z) return fail(SCW_ERR_ARG, "geev_mixed: the FP32 QR work must follow slot S1");
    const unsigned gZ = std::min<long long>(nblk(nn), 2048);
    const size_t cl_smem = (size_t)n * (sizeof(double2) + 4 * sizeof(int));
    const size_t eig_smem = 3 * sizeof(double2) * kMaxCluster * kMaxCluster;
    const size_t rot_smem = sizeof(double2) * (kMaxCluster * kMaxCluster + kMaxCluster * kMaxCluster);
    MX_TRY(set_smem((const void*)cluster_kernel, cl_smem));
    MX_TRY(set_smem((const void*)cluster_eig_kernel, eig_smem));
    MX_TRY(set_smem((const void*)rotate_kernel, rot_smem));
    const int maxcl = std::max(1, n / 2);
    const float2 f1 = {1.f, 0.f}, f0 = {0.f, 0.f};
    const double2 d1 = {1.0, 0.0}, d0 = {0.0, 0.0};
    double2* AX = reinterpret_cast<double2*>(w.S0);      // S0 and S1 together: one FP64 slot

    norm1_kernel<<<Z, 256, 0, st>>>(A, n, w.anorm);
    to_f32_kernel<<<nblk(nn * Z), 256, 0, st>>>(A, w.S0, nn * Z);
    MX_LAUNCHED(2);
    // FP32 Householder + QR + triangular eigenvectors: eigenvectors into S2, eigenvalues lam32
    MX_TRY(geev<float2>(st, w.S0, w.lam32, w.S2, n, Z, w.S1, w.qr, nullptr, prm.wide));
    if (launches) *launches += 5;
    init_kernel<<<dim3(gZ, Z), 256, 0, st>>>(w.lam32, w.S2, lam, V, n, w.qr, w.state, w.steps, w.res);
    cluster_kernel<<<Z, 1024, cl_smem, st>>>(lam, n, w.anorm, prm.tau_rel, w.label, w.member, w.cstart, w.ncl, w.state);
    MX_LAUNCHED(2);
    const int last = n >= EigMixParams::kLargeN ? std::max(prm.steps, prm.steps_large) : prm.steps;
    for (int s = 0; s <= last; s++) {
        // residual check (and right-hand side of the correction)
        MX_TRY(gemm<double2>(st, n, n, n, d1, A, n, nn, V, n, nn, d0, AX, n, nn, Z, w.state));
        resid_kernel<<<dim3((n + 31) / 32, Z), 256, 0, st>>>(AX, V, lam, n, w.S3, w.rn, w.xn, w.state);
        gate_kernel<<<Z, 256, 0, st>>>(n, w.rn, w.xn, w.anorm, s >= prm.steps ? prm.tol_accept : prm.tol, s, w.state,
                                       w.steps, w.res);
        MX_LAUNCHED(3);
        if (s == last) break;
        // E = X^-1 R in FP32
        to32_kernel<<<dim3(gZ, Z), 256, 0, st>>>(V, w.S0, w.S2, n, w.state);
        MX_LAUNCHED(1);
        MX_TRY(getrf<float2>(st, w.S0, n, nn, w.piv, n, w.info, Z));
        MX_TRY(getrs<float2>(st, w.S0, n, nn, w.piv, n, w.S3, n, nn, Z));
        if (launches) *launches += 3 * ((n + 31) / 32) + 1 + 4 * ((n + 63) / 64);
        lu_check_kernel<<<nblk(Z), 256, 0, st>>>(w.info, Z, w.state);
        singleton_kernel<<<dim3(nblk(n), Z), 256, 0, st>>>(w.S3, w.label, lam, n, w.state);
        cluster_eig_kernel<<<dim3(maxcl, Z), kMaxCluster, eig_smem, st>>>(w.S3, w.member, w.cstart, w.ncl, lam, n,
                                                                         w.anorm, prm.deg_rel, w.Y, w.state);
        f_kernel<<<dim3(gZ, Z), 256, 0, st>>>(w.S3, lam, w.label, n, w.S1, w.state);
        MX_LAUNCHED(4);
        // X += X F (FP32 product, FP64 sum), then the cluster rotations
        MX_TRY(gemm<float2>(st, n, n, n, f1, w.S2, n, nn, w.S1, n, nn, f0, w.S0, n, nn, Z, w.state));
        xupdate_kernel<<<dim3(gZ, Z), 256, 0, st>>>(w.S0, V, n, w.state);
        rotate_kernel<<<dim3(maxcl, Z), kMaxCluster, rot_smem, st>>>(V, w.member, w.cstart, w.ncl, w.Y, n, w.state);
        MX_LAUNCHED(3);
    }
    // slices without convergence: the FP64 Householder + QR solver (qr[] reused as the skip mask)
    final_kernel<<<nblk(Z), 256, 0, st>>>(w.state, w.qr, Z);
    MX_LAUNCHED(1);
    MX_TRY(geev<double2>(st, A, lam, V, n, Z, fb_work, status, w.qr, prm.wide));
    if (launches) *launches += 5;
    return SCW_OK;
}

}  // namespace mx
}  // namespace scw

// ------------------------------------------------------------------------------------
// C ABI: the mixed-precision eigen-solver on device buffers (a batched replacement of the
// reference's MKL_eigensolve, third_Lapack.h:38-47)
// ------------------------------------------------------------------------------------
extern "C" scw_status scw_zgeev_mixed(scw_ctx ctx, int n, void* A, void* W, void* V, int batch, int* accepted_host,
                                      int* steps_host, double* residual_host) {
    using namespace scw;
    if (!ctx || !A || !W || !V || n < 1 || batch < 1) return fail(SCW_ERR_ARG, "scw_zgeev_mixed: bad arguments");
    if (n > mx::kMaxN) return fail(SCW_ERR_ARG, "scw_zgeev_mixed: n above 4096");
    SCW_ON_DEVICE(ctx->device);
    const size_t nn = (size_t)n * n;
    // FP64 fallback work (>= 2 Z n^2 + 4 Z n float2 for S0, S1, hw, lam32), W region (S2, S3), small buffers
    const size_t pbytes = sizeof(double2) * (nn + 3 * (size_t)n) * batch;
    const size_t wbytes = sizeof(double2) * nn * batch;
    const size_t sbytes = mx::eigmix_small_bytes(n, batch);
    char* blk = nullptr;
    int* dst = nullptr;
    const size_t pal = (pbytes + 255) / 256 * 256, wal = (wbytes + 255) / 256 * 256;
    if (cudaMalloc(&blk, pal + wal + sbytes) != cudaSuccess || cudaMalloc(&dst, sizeof(int) * batch) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(blk);
        return fail(SCW_ERR_NOMEM, "scw_zgeev_mixed: workspace");
    }
    mx::EigMixWs w{};
    mx::eigmix_carve_small(w, blk + pal + wal, n, batch);
    float2* Pf = reinterpret_cast<float2*>(blk);
    float2* Wf = reinterpret_cast<float2*>(blk + pal);
    w.S0 = Pf;
    w.S1 = Pf + nn * batch;
    w.hw = Pf + 2 * nn * batch;
    w.lam32 = w.hw + 3 * (size_t)n * batch;
    w.S2 = Wf;
    w.S3 = Wf + nn * batch;
    long long L = 0;
    mx::EigMixParams prm;
    prm.wide = true;
    scw_status st = mx::geev_mixed(ctx->stream, (double2*)A, (double2*)W, (double2*)V, n, batch, w,
                                   reinterpret_cast<double2*>(blk), dst, prm, &L);
    ctx->launches += L;
    std::vector<int> status(batch, 0), state(batch, 0), steps(batch, 0);
    std::vector<double> res(batch, 0.0);
    if (st == SCW_OK) {
        cudaError_t e = cudaMemcpyAsync(status.data(), dst, sizeof(int) * batch, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(state.data(), w.state, sizeof(int) * batch, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(steps.data(), w.steps, sizeof(int) * batch, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(res.data(), w.res, sizeof(double) * batch, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) st = fail(SCW_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaFree(blk);
    cudaFree(dst);
    if (st != SCW_OK) return st;
    int bad = 0;
    for (int b = 0; b < batch; b++) {
        if (accepted_host) accepted_host[b] = state[b];
        if (steps_host) steps_host[b] = steps[b];
        if (residual_host) residual_host[b] = res[b];
        if (status[b]) bad = 1;
    }
    return bad ? fail(SCW_ERR_NUMERIC, "scw_zgeev_mixed: QR iteration did not converge") : SCW_OK;
}
