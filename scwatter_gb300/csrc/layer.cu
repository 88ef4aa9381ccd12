// Homogeneous multilayer solve (the reference program sCWatterLayer, sCWatterLayer.cpp:119-267)
// for a batch of incident plane waves on the GPU: per wave the 6L x 6L system of the
// transmitted / reflected amplitudes of every layer (rows: incident field and the absence of a
// wave entering from below, the transversality of every wave, and the four tangential
// continuity conditions at every interface), built in shared memory and solved by Gaussian
// elimination with partial pivoting -- one CTA per incident wave.
#include <cmath>
#include <vector>

#include "scw_internal.h"

namespace scw {
namespace ly {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, d = b.x + b.y * r;
        return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    }
    const double r = b.x / b.y, d = b.x * r + b.y;
    return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
__device__ __forceinline__ double cabs1(double2 a) { return fabs(a.x) + fabs(a.y); }
__device__ __forceinline__ double2 cexp_i(double2 a) {      // exp(i a)
    const double m = exp(-a.y);
    double s, c;
    sincos(a.x, &s, &c);
    return make_double2(m * c, m * s);
}
__device__ __forceinline__ double2 csqrt_p(double2 a) {     // principal square root
    if (a.x == 0.0 && a.y == 0.0) return make_double2(0.0, 0.0);
    const double t = sqrt(0.5 * (fabs(a.x) + hypot(a.x, a.y)));
    if (a.x >= 0.0) return make_double2(t, a.y / (2.0 * t));
    return make_double2(fabs(a.y) / (2.0 * t), copysign(t, a.y));
}

// waves: per wave 12 doubles (E0 xyz re/im, k xyz re/im); ri: L complex indices;
// z: L-1 interfaces; x: per wave 6L complex (layer l: T xyz then R xyz)
__global__ void layer_kernel(const double* __restrict__ waves, int L, const double2* __restrict__ ri,
                             const double* __restrict__ z, double n0, double k, double2* __restrict__ x,
                             int* __restrict__ info) {
    extern __shared__ double2 sm[];
    const int N = 6 * L;
    double2* A = sm;                 // N x N
    double2* b = A + N * N;          // N
    double2* sz = b + N;             // L
    __shared__ double s_dir[3];
    __shared__ int s_piv;
    const int w = blockIdx.x;
    const double* pw = waves + 12 * (long long)w;
    if (threadIdx.x == 0) {
        // direction = Re k / |Re k| (the planewave's propagation direction)
        const double kx = pw[6], ky = pw[8], kz = pw[10];
        const double nk = sqrt(kx * kx + ky * ky + kz * kz);
        s_dir[0] = kx / nk;
        s_dir[1] = ky / nk;
        s_dir[2] = kz / nk;
    }
    for (int e = threadIdx.x; e < N * N; e += blockDim.x) A[e] = make_double2(0.0, 0.0);
    for (int e = threadIdx.x; e < N; e += blockDim.x) b[e] = make_double2(0.0, 0.0);
    __syncthreads();
    const double sx = s_dir[0], sy = s_dir[1];
    // InitSz: sz_l = sqrt(ri_l^2 - (n0 s_x)^2 - (n0 s_y)^2)
    for (int l = threadIdx.x; l < L; l += blockDim.x) {
        const double2 r = ri[l];
        const double2 r2 = cmul(r, r);
        sz[l] = csqrt_p(make_double2(r2.x - (sx * n0) * (sx * n0) - (sy * n0) * (sy * n0), r2.y));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        auto M = [&](int row, int layer, int dir, int c) -> double2& { return A[row * N + layer * 6 + dir * 3 + c]; };
        // boundary conditions (SetBoundaryConditions)
        M(0, 0, 0, 0) = make_double2(1, 0);
        M(1, 0, 0, 1) = make_double2(1, 0);
        M(2, 0, 0, 2) = make_double2(1, 0);
        b[0] = make_double2(pw[0], pw[1]);
        b[1] = make_double2(pw[2], pw[3]);
        b[2] = make_double2(pw[4], pw[5]);
        M(3, L - 1, 1, 0) = make_double2(1, 0);
        M(4, L - 1, 1, 1) = make_double2(1, 0);
        M(5, L - 1, 1, 2) = make_double2(1, 0);
        // transversality (SetGaussianConstraints): direction s without the n0 factor, sz with it
        int start = 6;
        for (int l = 0; l < L - 1; l++) {
            M(start + l, l, 1, 0) = make_double2(sx, 0);
            M(start + l, l, 1, 1) = make_double2(sy, 0);
            M(start + l, l, 1, 2) = make_double2(-sz[l].x, -sz[l].y);
        }
        start += L - 2;
        for (int l = 1; l < L; l++) {
            M(start + l, l, 0, 0) = make_double2(sx, 0);
            M(start + l, l, 0, 1) = make_double2(sy, 0);
            M(start + l, l, 0, 2) = sz[l];
        }
        // interface continuity (SetBoundaryConstraints)
        start = 6 + 2 * (L - 1);
        for (int l = 0; l < L - 1; l++) {
            const double zn = (l == 0) ? z[l] : z[l] - z[l - 1];
            const double zp = (l == L - 2) ? 0.0 : z[l] - z[l + 1];
            const double2 en = cexp_i(make_double2(k * sz[l].x * zn, k * sz[l].y * zn));                 // exp(i k sz_l zn)
            const double2 ep = cexp_i(make_double2(-k * sz[l + 1].x * zp, -k * sz[l + 1].y * zp));       // exp(-i k sz_{l+1} zp)
            const double2 one = make_double2(1, 0), mone = make_double2(-1, 0);
            const double2 nep = make_double2(-ep.x, -ep.y);
            const int r0 = start + 4 * l;
            M(r0, l, 0, 0) = en;
            M(r0, l, 1, 0) = one;
            M(r0, l + 1, 0, 0) = mone;
            M(r0, l + 1, 1, 0) = nep;
            M(r0 + 1, l, 0, 1) = en;
            M(r0 + 1, l, 1, 1) = one;
            M(r0 + 1, l + 1, 0, 1) = mone;
            M(r0 + 1, l + 1, 1, 1) = nep;
            const double2 szl = sz[l], szl1 = sz[l + 1];
            M(r0 + 2, l, 0, 2) = make_double2(sy * en.x, sy * en.y);
            M(r0 + 2, l, 0, 1) = make_double2(-cmul(szl, en).x, -cmul(szl, en).y);
            M(r0 + 2, l, 1, 2) = make_double2(sy, 0);
            M(r0 + 2, l, 1, 1) = szl;
            M(r0 + 2, l + 1, 0, 2) = make_double2(-sy, 0);
            M(r0 + 2, l + 1, 0, 1) = szl1;
            M(r0 + 2, l + 1, 1, 2) = make_double2(-sy * ep.x, -sy * ep.y);
            M(r0 + 2, l + 1, 1, 1) = make_double2(-cmul(szl1, ep).x, -cmul(szl1, ep).y);
            M(r0 + 3, l, 0, 0) = cmul(szl, en);
            M(r0 + 3, l, 0, 2) = make_double2(-sx * en.x, -sx * en.y);
            M(r0 + 3, l, 1, 0) = make_double2(-szl.x, -szl.y);
            M(r0 + 3, l, 1, 2) = make_double2(-sx, 0);
            M(r0 + 3, l + 1, 0, 0) = make_double2(-szl1.x, -szl1.y);
            M(r0 + 3, l + 1, 0, 2) = make_double2(sx, 0);
            M(r0 + 3, l + 1, 1, 0) = cmul(szl1, ep);
            M(r0 + 3, l + 1, 1, 2) = make_double2(sx * ep.x, sx * ep.y);
        }
    }
    __syncthreads();
    // Gaussian elimination with partial pivoting
    int singular = 0;
    for (int c = 0; c < N; c++) {
        if (threadIdx.x == 0) {
            int p = c;
            double best = cabs1(A[c * N + c]);
            for (int r = c + 1; r < N; r++) {
                const double v = cabs1(A[r * N + c]);
                if (v > best) {
                    best = v;
                    p = r;
                }
            }
            s_piv = best > 0.0 ? p : -1;
        }
        __syncthreads();
        const int p = s_piv;
        if (p < 0) {
            singular = 1;
            break;
        }
        if (p != c) {
            for (int j = threadIdx.x; j < N; j += blockDim.x) {
                const double2 t = A[c * N + j];
                A[c * N + j] = A[p * N + j];
                A[p * N + j] = t;
            }
            if (threadIdx.x == 0) {
                const double2 t = b[c];
                b[c] = b[p];
                b[p] = t;
            }
        }
        __syncthreads();
        const double2 piv = A[c * N + c];
        for (int r = c + 1 + threadIdx.x; r < N; r += blockDim.x) {
            const double2 m = cdiv(A[r * N + c], piv);
            if (m.x == 0.0 && m.y == 0.0) continue;
            for (int j = c + 1; j < N; j++) A[r * N + j] = csub(A[r * N + j], cmul(m, A[c * N + j]));
            b[r] = csub(b[r], cmul(m, b[c]));
            A[r * N + c] = make_double2(0.0, 0.0);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        info[w] = singular;
        double2* xw = x + (long long)w * N;
        if (!singular) {
            for (int r = N - 1; r >= 0; r--) {
                double2 s = b[r];
                for (int j = r + 1; j < N; j++) s = csub(s, cmul(A[r * N + j], xw[j]));
                xw[r] = cdiv(s, A[r * N + r]);
            }
        }
    }
}

}  // namespace ly
}  // namespace scw

using scw::fail;

extern "C" {

// sCWatterLayer's system for `count` incident plane waves (HOST records of 12 doubles each):
// ri = L complex refractive indices (layer 0 is the incident medium), z = L - 1 interface
// positions, n0 = Re ri[0] (the reference scales the direction by it), k = vacuum wavenumber.
// x (HOST, count x 6L complex): per layer T xyz then R xyz; info (HOST, count ints): 1 if the
// system was singular.
scw_status scw_layer_solve(scw_ctx ctx, int L, const double* ri, const double* z, double n0, double k, int count,
                           const double* waves, double* x, int* info) {
    if (!ctx || L < 2 || L > 16 || !ri || !z || count < 1 || !waves || !x || !info)
        return fail(SCW_ERR_ARG, "scw_layer_solve: bad arguments (2 <= L <= 16)");
    SCW_ON_DEVICE(ctx->device);
    const int N = 6 * L;
    // sub-buffers at 256-byte offsets (double2 needs 16-byte alignment whatever L is)
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t o_z = al(sizeof(double2) * L), o_w = o_z + al(sizeof(double) * (L - 1)),
                 o_x = o_w + al(sizeof(double) * 12 * (size_t)count), o_i = o_x + al(sizeof(double2) * (size_t)N * count);
    scw::DevBuf buf;
    scw_status st = buf.reserve(o_i + al(sizeof(int) * count));
    if (st != SCW_OK) return st;
    char* p = (char*)buf.ptr;
    double2* d_ri = (double2*)p;
    double* d_z = (double*)(p + o_z);
    double* d_w = (double*)(p + o_w);
    double2* d_x = (double2*)(p + o_x);
    int* d_info = (int*)(p + o_i);
    cudaStream_t s = ctx->stream;
    SCW_CUDA_TRY(cudaMemcpyAsync(d_ri, ri, sizeof(double2) * L, cudaMemcpyHostToDevice, s));
    SCW_CUDA_TRY(cudaMemcpyAsync(d_z, z, sizeof(double) * (L - 1), cudaMemcpyHostToDevice, s));
    SCW_CUDA_TRY(cudaMemcpyAsync(d_w, waves, sizeof(double) * 12 * (size_t)count, cudaMemcpyHostToDevice, s));
    const size_t smem = sizeof(double2) * ((size_t)N * N + N + L);
    SCW_CUDA_TRY(cudaFuncSetAttribute(scw::ly::layer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    scw::ly::layer_kernel<<<count, 128, smem, s>>>(d_w, L, d_ri, d_z, n0, k, d_x, d_info);
    SCW_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    SCW_CUDA_TRY(cudaMemcpyAsync(x, d_x, sizeof(double2) * (size_t)N * count, cudaMemcpyDeviceToHost, s));
    SCW_CUDA_TRY(cudaMemcpyAsync(info, d_info, sizeof(int) * count, cudaMemcpyDeviceToHost, s));
    SCW_CUDA_TRY(cudaStreamSynchronize(s));
    buf.release();
    return SCW_OK;
}

}  // extern "C"
