// Warm-started eigensolver for batches of n x n complex matrices (the layers' PQ).
//
// Given one proposed shift per eigenvalue (from the learned model, or any other guess), each
// eigenpair is found independently by Rayleigh-quotient iteration on the Hessenberg form H of
// the matrix (A = Q H Q^H):
//   factor (H - sigma I) by Gaussian elimination with pivoting between adjacent rows (O(n^2),
//   the Hessenberg structure leaves one row to eliminate per column), solve, normalise,
//   after two solves with the proposed shift sigma <- x^H H x, until ||H x - sigma x|| stops
//   decreasing or falls below 1e-14 ||H||.
// One warp owns one (matrix, eigenvalue) task; tasks of all matrices run concurrently, so the
// sequential QR sweeps of the plain eigen-solver are replaced by n independent O(n^2) chains.
// A matrix is accepted only when
//   * every eigenpair has ||A v - lambda v|| <= tol ||A||_F ||v|| (checked against A itself), and
//   * the mode count is intact: no two eigenpairs converged to the same eigenvector
//     (eigenvalues within 1e-7 |lambda|_max of each other whose vectors overlap by > 0.5);
// A task that converged onto another task's eigenvector is restarted with that eigenvector (and
// the ones it met before) projected out of its first iterates, for a few rounds; a matrix still
// failing a gate falls back to the plain eigen-solver (zgeev), whose result replaces it.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "scw_dense.h"

namespace scw {
namespace wm {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {   // conj(a) b
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
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
__device__ __forceinline__ double2 warp_sum(double2 v) {
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}
__device__ __forceinline__ double warp_sumd(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__host__ __device__ __forceinline__ long long row_off(int k, int n) {   // packed upper rows: row k holds cols k..n-1
    return (long long)k * n - (long long)k * (k - 1) / 2;
}

// ||H||_F per matrix (one block per matrix)
__global__ void fro_kernel(const double2* __restrict__ A, int n, double* __restrict__ out) {
    const double2* a = A + (long long)blockIdx.x * n * n;
    double s = 0.0;
    for (long long e = threadIdx.x; e < (long long)n * n; e += blockDim.x) s += a[e].x * a[e].x + a[e].y * a[e].y;
    __shared__ double sh[32];
    s = warp_sumd(s);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
        out[blockIdx.x] = sqrt(t);
    }
}

constexpr int kFixed = 2;   // solves with the proposed shift before the Rayleigh quotient takes over
constexpr int kMaxExcl = 8; // eigenvectors a repair task projects out
constexpr int kRepairRounds = 8;

// y <- y - sum_e v_e (v_e^H y) for the excluded unit eigenvectors (columns of Xold)
__device__ void project_out(double2* y, const double2* Xb, const int* ex, int n, int lane) {
    for (int e = 0; e < kMaxExcl; e++) {
        const int c = ex[e];
        if (c < 0) break;
        double2 d = make_double2(0.0, 0.0);
        for (int i = lane; i < n; i += 32) d = cadd(d, cmulc(Xb[(long long)i * n + c], y[i]));
        d = warp_sum(d);
        __syncwarp();
        for (int i = lane; i < n; i += 32) y[i] = csub(y[i], cmul(Xb[(long long)i * n + c], d));
        __syncwarp();
    }
}

// Rayleigh-quotient iteration, one warp per task t = task0 + warp (matrix t / n, eigenvalue t % n).
__global__ void __launch_bounds__(128)
rqi_kernel(const double2* __restrict__ H, int n, const double2* __restrict__ shifts, const double* __restrict__ hnorm,
           double2* __restrict__ ws, long long ws_stride, long long task0, long long ntasks, int max_it,
           double2* __restrict__ lam_out, double2* __restrict__ X, int* __restrict__ iters,
           const long long* __restrict__ task_ids, const int* __restrict__ excl, const double2* __restrict__ Xold,
           const double2* __restrict__ Qm, const int* __restrict__ start_idx) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= ntasks) return;
    const long long t = task_ids ? task_ids[task0 + w] : task0 + w;
    const int* ex = excl ? excl + (task0 + w) * kMaxExcl : nullptr;
    const long long b = t / n;
    const int j = (int)(t % n);
    const double2* Hb = H + b * (long long)n * n;
    double2* U = ws + w * ws_stride;
    double2* x = U + row_off(n, n);
    double2* y = x + n;
    const double hn = fmax(hnorm[b], 1e-300);
    const double tiny = 2.220446049250313e-16 * hn;
    // start vector: Q^H e_s for a proposed mode s (row s of Q, conjugated: a unit vector), or a
    // deterministic pseudo-random unit vector per task
    const int s0 = start_idx ? start_idx[t] : -1;
    double ss = 0;
    if (s0 >= 0 && s0 < n) {
        const double2* qrow = Qm + b * (long long)n * n + (long long)s0 * n;
        for (int i = lane; i < n; i += 32) {
            const double2 q = qrow[i];
            x[i] = make_double2(q.x, -q.y);
            ss += q.x * q.x + q.y * q.y;
        }
    } else
    for (int i = lane; i < n; i += 32) {
        unsigned h = (unsigned)(i * 2654435761u) ^ (unsigned)(j * 2246822519u) ^ 0x9e3779b9u;
        h ^= h >> 15;
        h *= 2246822519u;
        h ^= h >> 13;
        const double a = 0.5 + (double)(h & 0xffff) / 65536.0, c = (double)((h >> 16) & 0xffff) / 65536.0 - 0.5;
        x[i] = make_double2(a, c);
        ss += a * a + c * c;
    }
    ss = warp_sumd(ss);
    const double inv0 = 1.0 / sqrt(ss);
    for (int i = lane; i < n; i += 32) x[i] = make_double2(x[i].x * inv0, x[i].y * inv0);
    __syncwarp();
    if (ex) project_out(x, Xold + b * (long long)n * n, ex, n, lane);
    double2 sigma = shifts[t];
    double2 lam_fin = sigma;
    const int nfix = s0 >= 0 ? 1 : kFixed;
    double best = 1e300;
    int it = 0;
    for (; it < max_it; it++) {
        // ---- factor (H - sigma I) row by row, eliminating the rhs (copy of x) on the fly ----
        for (int i = lane; i < n; i += 32) y[i] = x[i];
        for (int c = lane; c < n; c += 32) {
            double2 v = Hb[c];
            if (c == 0) v = csub(v, sigma);
            U[c] = v;
        }
        __syncwarp();
        for (int k = 0; k + 1 < n; k++) {
            const long long ok = row_off(k, n), ok1 = row_off(k + 1, n);
            const double2 wk = U[ok];
            const double2 rk = Hb[(long long)(k + 1) * n + k];
            const bool piv = cabs1(rk) > cabs1(wk);
            double2 m = make_double2(0.0, 0.0);
            if (piv) m = cdiv(wk, rk);
            else if (cabs1(wk) > 0.0) m = cdiv(rk, wk);
            for (int c = k + 1 + lane; c < n; c += 32) {
                const double2 wc = U[ok + (c - k)];
                double2 rc = Hb[(long long)(k + 1) * n + c];
                if (c == k + 1) rc = csub(rc, sigma);
                if (piv) {
                    U[ok + (c - k)] = rc;
                    U[ok1 + (c - k - 1)] = csub(wc, cmul(m, rc));
                } else {
                    U[ok1 + (c - k - 1)] = csub(rc, cmul(m, wc));
                }
            }
            if (lane == 0) {
                const double2 yk = y[k], yk1 = y[k + 1];
                if (piv) {
                    U[ok] = rk;
                    y[k] = yk1;
                    y[k + 1] = csub(yk, cmul(m, yk1));
                } else {
                    y[k + 1] = csub(yk1, cmul(m, yk));
                }
            }
            __syncwarp();
        }
        // ---- back substitution (zero pivots perturbed to eps ||H||, as inverse iteration does) ----
        for (int k = n - 1; k >= 0; k--) {
            const long long ok = row_off(k, n);
            double2 s = make_double2(0.0, 0.0);
            for (int c = k + 1 + lane; c < n; c += 32) s = cadd(s, cmul(U[ok + (c - k)], y[c]));
            s = warp_sum(s);
            if (lane == 0) {
                double2 d = U[ok];
                if (cabs1(d) < tiny) d = make_double2(tiny, 0.0);
                y[k] = cdiv(csub(y[k], s), d);
            }
            __syncwarp();
        }
        if (ex && it < nfix) project_out(y, Xold + b * (long long)n * n, ex, n, lane);
        // ---- normalise, Rayleigh quotient and residual ----
        double nn2 = 0;
        for (int i = lane; i < n; i += 32) nn2 += y[i].x * y[i].x + y[i].y * y[i].y;
        nn2 = warp_sumd(nn2);
        if (!(nn2 > 0.0) || !isfinite(nn2)) break;
        const double inv = 1.0 / sqrt(nn2);
        for (int i = lane; i < n; i += 32) x[i] = make_double2(y[i].x * inv, y[i].y * inv);
        __syncwarp();
        // hx = H x into y; rq = x^H H x
        double2 rq = make_double2(0.0, 0.0);
        for (int i = 0; i < n; i++) {
            double2 s = make_double2(0.0, 0.0);
            const double2* row = Hb + (long long)i * n;
            for (int c = max(i - 1, 0) + lane; c < n; c += 32) s = cadd(s, cmul(row[c], x[c]));
            s = warp_sum(s);
            if (lane == 0) y[i] = s;
            rq = cadd(rq, cmulc(x[i], s));
        }
        __syncwarp();
        double r2 = 0;
        for (int i = lane; i < n; i += 32) {
            const double2 d = csub(y[i], cmul(rq, x[i]));
            r2 += d.x * d.x + d.y * d.y;
        }
        r2 = warp_sumd(r2);
        const double r = sqrt(r2);
        lam_fin = rq;
        if (r <= 1e-14 * hn) {
            it++;
            break;
        }
        if (it >= nfix + 1 && r <= 1e-10 * hn && r > 0.5 * best) {   // stagnation at rounding level
            it++;
            break;
        }
        // the first solves keep the proposed shift (inverse iteration locks onto the eigenvector
        // nearest to it; one solve when the start vector is a proposed mode, kFixed otherwise);
        // then the Rayleigh quotient becomes the shift
        if (it + 1 >= nfix) sigma = rq;
        best = fmin(best, r);
    }
    for (int i = lane; i < n; i += 32) X[b * (long long)n * n + (long long)i * n + j] = x[i];
    if (lane == 0) {
        lam_out[t] = lam_fin;
        iters[t] = it;
    }
}

// R = A V - V diag(lambda): per column relative residual; per matrix the maximum (as an
// ordered int of the double bits, for atomicMax)
__global__ void resid_kernel(const double2* __restrict__ AV, const double2* __restrict__ V,
                             const double2* __restrict__ lam, const double* __restrict__ anorm, int n,
                             unsigned long long* __restrict__ worst) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;    // column task
    const long long b = blockIdx.y;
    if (t >= n) return;
    const double2* av = AV + b * (long long)n * n;
    const double2* v = V + b * (long long)n * n;
    const double2 l = lam[b * n + t];
    double r2 = 0, v2 = 0;
    for (int i = 0; i < n; i++) {
        const double2 vi = v[(long long)i * n + t];
        const double2 d = csub(av[(long long)i * n + t], cmul(l, vi));
        r2 += d.x * d.x + d.y * d.y;
        v2 += vi.x * vi.x + vi.y * vi.y;
    }
    const double rel = sqrt(r2) / (fmax(anorm[b], 1e-300) * fmax(sqrt(v2), 1e-300));
    const double val = isfinite(rel) ? rel : 1e300;
    atomicMax(worst + b, (unsigned long long)__double_as_longlong(val));
}

// mode count: pairs (i < k) of nearly equal eigenvalues whose eigenvectors overlap; dup_of[k]
// receives the smallest such i
__global__ void dup_kernel(const double2* __restrict__ lam, const double2* __restrict__ V, int n, double rel,
                           int* __restrict__ dup, int* __restrict__ dup_of) {
    const long long b = blockIdx.y;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (long long)n * n) return;
    const int i = (int)(p / n), k = (int)(p % n);
    if (k <= i) return;
    const double2* l = lam + b * n;
    double scale = 0;
    // |lambda|_max is approximated by the larger of the two: duplicates sit at the same value
    scale = fmax(cabs1(l[i]), cabs1(l[k]));
    if (cabs1(csub(l[i], l[k])) > rel * fmax(scale, 1e-300)) return;
    const double2* v = V + b * (long long)n * n;
    double2 o = make_double2(0.0, 0.0);
    double ni = 0, nk = 0;
    for (int r = 0; r < n; r++) {
        const double2 a = v[(long long)r * n + i], c = v[(long long)r * n + k];
        o = cadd(o, cmulc(a, c));
        ni += a.x * a.x + a.y * a.y;
        nk += c.x * c.x + c.y * c.y;
    }
    if (sqrt(o.x * o.x + o.y * o.y) > 0.5 * sqrt(ni * nk)) {
        atomicExch(dup + b, 1);
        atomicMin(dup_of + b * n + k, i);
    }
}

static unsigned blocks(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace wm
}  // namespace scw

using scw::fail;

extern "C" {

// A: device, batch x n x n complex128 (not modified); shifts: device, batch x n complex128;
// start_idx: device, batch x n ints (a proposed mode per eigenpair: the start vector is that
// unit vector of A's basis; -1 or NULL: pseudo-random start).
// W (batch x n) and V (batch x n x n, column k = eigenvector k): device outputs.
// accepted_host[b] = 1 when matrix b passed the gates (0: it was solved by the plain eigen-solver).
// stats_host (may be NULL): [0] mean Rayleigh iterations per eigenpair, [1] largest accepted
// relative residual, [2] matrices accepted, [3] matrices that fell back, [4] repaired tasks.
scw_status scw_eig_warm(scw_ctx ctx, int n, const void* A_, int batch, const void* shifts_, const int* start_idx,
                        int max_it, double tol, void* W_, void* V_, int* accepted_host, double* stats_host) {
    using namespace scw::wm;
    if (!ctx || n < 1 || !A_ || batch < 1 || !shifts_ || !W_ || !V_ || max_it < 1 || !(tol > 0))
        return fail(SCW_ERR_ARG, "scw_eig_warm: bad arguments");
    SCW_ON_DEVICE(ctx->device);
    cudaStream_t st = ctx->stream;
    const double2* A = (const double2*)A_;
    const double2* shifts = (const double2*)shifts_;
    double2* W = (double2*)W_;
    double2* V = (double2*)V_;
    const long long nn = (long long)n * n;
    // workspace: H, Q, X, AV (batch nn each), hessenberg work (batch 3n), norms, flags
    scw::DevBuf buf;
    const size_t base = sizeof(double2) * (size_t)(5 * nn * batch + 3LL * n * batch) + sizeof(double) * 2 * batch +
                        sizeof(unsigned long long) * batch + sizeof(int) * (batch + 2 * (size_t)n * batch) +
                        (sizeof(long long) + sizeof(int) * kMaxExcl) * (size_t)n * batch + 8192;
    scw_status s = buf.reserve(base);
    if (s != SCW_OK) return s;
    char* p = (char*)buf.ptr;
    auto take = [&](size_t bytes) {
        char* r = p;
        p += (bytes + 255) / 256 * 256;
        return r;
    };
    double2* Hm = (double2*)take(sizeof(double2) * nn * batch);
    double2* Qm = (double2*)take(sizeof(double2) * nn * batch);
    double2* Xm = (double2*)take(sizeof(double2) * nn * batch);
    double2* AV = (double2*)take(sizeof(double2) * nn * batch);
    double2* hw = (double2*)take(sizeof(double2) * 3 * (size_t)n * batch);
    double* hnorm = (double*)take(sizeof(double) * batch);
    double* anorm = (double*)take(sizeof(double) * batch);
    unsigned long long* worst = (unsigned long long*)take(sizeof(unsigned long long) * batch);
    int* dup = (int*)take(sizeof(int) * batch);
    int* iters = (int*)take(sizeof(int) * (size_t)n * batch);
    double2* Xold = (double2*)take(sizeof(double2) * nn * batch);
    int* dup_of = (int*)take(sizeof(int) * (size_t)n * batch);
    long long* rep_ids = (long long*)take(sizeof(long long) * (size_t)n * batch);
    int* rep_excl = (int*)take(sizeof(int) * kMaxExcl * (size_t)n * batch);
    // Hessenberg form and its norm
    SCW_CUDA_TRY(cudaMemcpyAsync(Hm, A, sizeof(double2) * nn * batch, cudaMemcpyDeviceToDevice, st));
    s = scw::zgehrd(st, Hm, Qm, n, batch, hw);
    if (s != SCW_OK) return s;
    fro_kernel<<<batch, 256, 0, st>>>(Hm, n, hnorm);
    fro_kernel<<<batch, 256, 0, st>>>(A, n, anorm);
    SCW_CUDA_TRY(cudaGetLastError());
    // Rayleigh-quotient tasks in chunks bounded by the factor storage (packed n(n+1)/2 + 2n per task)
    const long long ws_stride = (row_off(n, n) + 2LL * n + 31) / 32 * 32;
    size_t free_b = 0, total_b = 0;
    SCW_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    const long long total = (long long)n * batch;
    long long chunk = std::max<long long>(4, std::min<long long>(total, (long long)(0.5 * free_b) /
                                                                           (ws_stride * (long long)sizeof(double2))));
    chunk = std::min<long long>(chunk, 152LL * 64);
    scw::DevBuf tw;
    if ((s = tw.reserve(sizeof(double2) * (size_t)ws_stride * chunk)) != SCW_OK) return s;
    long long launches = 4;
    auto run_tasks = [&](long long count, const long long* ids, const int* excl) -> scw_status {
        for (long long t0 = 0; t0 < count; t0 += chunk) {
            const long long cnt = std::min(chunk, count - t0);
            rqi_kernel<<<blocks(cnt * 32, 128), 128, 0, st>>>(Hm, n, shifts, hnorm, (double2*)tw.ptr, ws_stride, t0, cnt,
                                                              max_it, W, Xm, iters, ids, excl, Xold, Qm, start_idx);
            SCW_CUDA_TRY(cudaGetLastError());
            launches++;
        }
        return SCW_OK;
    };
    if ((s = run_tasks(total, nullptr, nullptr)) != SCW_OK) return s;
    std::vector<unsigned long long> hw_worst(batch);
    std::vector<int> hdup(batch), hdup_of((size_t)n * batch), hit((size_t)n * batch);
    std::vector<long long> rep_tasks;
    std::vector<int> rep_ex;
    std::vector<std::vector<int>> chain((size_t)n * batch);   // eigenvectors each task has to avoid
    int repairs = 0;
    for (int round = 0;; round++) {
        // back-transform V = Q X, residual against A, mode-count check
        s = scw::zgemm(st, n, n, n, make_double2(1, 0), Qm, n, nn, Xm, n, nn, make_double2(0, 0), V, n, nn, batch);
        if (s != SCW_OK) return s;
        s = scw::zgemm(st, n, n, n, make_double2(1, 0), A, n, nn, V, n, nn, make_double2(0, 0), AV, n, nn, batch);
        if (s != SCW_OK) return s;
        SCW_CUDA_TRY(cudaMemsetAsync(worst, 0, sizeof(unsigned long long) * batch, st));
        SCW_CUDA_TRY(cudaMemsetAsync(dup, 0, sizeof(int) * batch, st));
        SCW_CUDA_TRY(cudaMemsetAsync(dup_of, 0x7f, sizeof(int) * (size_t)n * batch, st));
        resid_kernel<<<dim3(blocks(n), batch), 256, 0, st>>>(AV, V, W, anorm, n, worst);
        dup_kernel<<<dim3(blocks(nn), batch), 256, 0, st>>>(W, V, n, 1e-7, dup, dup_of);
        SCW_CUDA_TRY(cudaGetLastError());
        launches += 4;
        SCW_CUDA_TRY(cudaMemcpyAsync(hw_worst.data(), worst, sizeof(unsigned long long) * batch, cudaMemcpyDeviceToHost, st));
        SCW_CUDA_TRY(cudaMemcpyAsync(hdup.data(), dup, sizeof(int) * batch, cudaMemcpyDeviceToHost, st));
        SCW_CUDA_TRY(cudaMemcpyAsync(hdup_of.data(), dup_of, sizeof(int) * hdup_of.size(), cudaMemcpyDeviceToHost, st));
        SCW_CUDA_TRY(cudaStreamSynchronize(st));
        if (round == kRepairRounds) break;
        // repair: a task that converged onto the eigenvector of a lower-numbered task restarts with
        // that eigenvector (and the ones it met before) projected out of its first iterates
        rep_tasks.clear();
        rep_ex.clear();
        for (int b = 0; b < batch; b++) {
            if (!hdup[b]) continue;
            for (int k = 0; k < n; k++) {
                const int i = hdup_of[(size_t)b * n + k];
                if (i < 0 || i >= n) continue;
                auto& ch = chain[(size_t)b * n + k];
                if ((int)ch.size() >= kMaxExcl) continue;
                if (std::find(ch.begin(), ch.end(), i) == ch.end()) ch.push_back(i);
                rep_tasks.push_back((long long)b * n + k);
                for (int e = 0; e < kMaxExcl; e++) rep_ex.push_back(e < (int)ch.size() ? ch[e] : -1);
            }
        }
        if (rep_tasks.empty()) break;
        repairs += (int)rep_tasks.size();
        SCW_CUDA_TRY(cudaMemcpyAsync(Xold, Xm, sizeof(double2) * nn * batch, cudaMemcpyDeviceToDevice, st));
        SCW_CUDA_TRY(cudaMemcpyAsync(rep_ids, rep_tasks.data(), sizeof(long long) * rep_tasks.size(),
                                     cudaMemcpyHostToDevice, st));
        SCW_CUDA_TRY(cudaMemcpyAsync(rep_excl, rep_ex.data(), sizeof(int) * rep_ex.size(), cudaMemcpyHostToDevice, st));
        if ((s = run_tasks((long long)rep_tasks.size(), rep_ids, rep_excl)) != SCW_OK) return s;
    }
    SCW_CUDA_TRY(cudaMemcpyAsync(hit.data(), iters, sizeof(int) * hit.size(), cudaMemcpyDeviceToHost, st));
    SCW_CUDA_TRY(cudaStreamSynchronize(st));
    std::vector<int> reject;
    double max_acc = 0;
    for (int b = 0; b < batch; b++) {
        double r;
        std::memcpy(&r, &hw_worst[b], sizeof(double));
        const bool ok = r <= tol && !hdup[b];
        if (accepted_host) accepted_host[b] = ok ? 1 : 0;
        if (ok) max_acc = std::max(max_acc, r);
        else reject.push_back(b);
    }
    // fallback: the plain eigen-solver on the rejected matrices
    if (!reject.empty()) {
        const int nr = (int)reject.size();
        scw::DevBuf fb;
        if ((s = fb.reserve(sizeof(double2) * ((size_t)nn * nr * 3 + (size_t)n * nr * 4) + sizeof(int) * nr + 1024)) !=
            SCW_OK)
            return s;
        double2* FA = (double2*)fb.ptr;
        double2* FV = FA + nn * nr;
        double2* FWk = FV + nn * nr;                 // work: nn + 3n per matrix
        double2* FW = FWk + (nn + 3LL * n) * nr;
        int* fst = (int*)(FW + (long long)n * nr);
        for (int i = 0; i < nr; i++)
            SCW_CUDA_TRY(cudaMemcpyAsync(FA + nn * i, A + nn * reject[i], sizeof(double2) * nn,
                                         cudaMemcpyDeviceToDevice, st));
        if ((s = scw::zgeev(st, FA, FW, FV, n, nr, FWk, fst)) != SCW_OK) return s;
        for (int i = 0; i < nr; i++) {
            SCW_CUDA_TRY(cudaMemcpyAsync(V + nn * reject[i], FV + nn * i, sizeof(double2) * nn, cudaMemcpyDeviceToDevice, st));
            SCW_CUDA_TRY(cudaMemcpyAsync(W + (long long)n * reject[i], FW + (long long)n * i, sizeof(double2) * n,
                                         cudaMemcpyDeviceToDevice, st));
        }
        std::vector<int> hst(nr);
        SCW_CUDA_TRY(cudaMemcpyAsync(hst.data(), fst, sizeof(int) * nr, cudaMemcpyDeviceToHost, st));
        SCW_CUDA_TRY(cudaStreamSynchronize(st));
        launches += 5;
        for (int v : hst)
            if (v) return fail(SCW_ERR_NUMERIC, "scw_eig_warm: the fallback eigen-solver did not converge");
    }
    ctx->launches += launches;
    if (stats_host) {
        double sum = 0;
        for (int v : hit) sum += v;
        stats_host[0] = sum / (double)hit.size();
        stats_host[1] = max_acc;
        stats_host[2] = (double)(batch - (int)reject.size());
        stats_host[3] = (double)reject.size();
        stats_host[4] = (double)repairs;
    }
    return SCW_OK;
}

}  // extern "C"
