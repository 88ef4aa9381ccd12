// Sample volumes on the device: the synthetic generators of the workloads and a .npy reader
// that streams the volume into device memory (the reference reads the sample on the host with
// tira's load_npy, FourierWave.h:269, and generates it with tilesample.py).  With these a
// batch or a solve never moves the sample volume through host memory.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "scw_internal.h"

using scw::fail;

namespace {

unsigned nblk(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// Spheres in order over a constant background; a voxel (z, y, x) is inside when
// (z - cz)^2 + (y - cy)^2 + (x - cx)^2 <= r^2 (the test of the host generator, same order)
__global__ void spheres_kernel(int Z, int Y, int X, int ns, const double* __restrict__ sph, double2 bg, double2 in,
                               double2* __restrict__ out) {
    const long long total = (long long)Z * Y * X;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % X), y = (int)((i / X) % Y), z = (int)(i / ((long long)X * Y));
        double2 v = bg;
        for (int s = 0; s < ns; s++) {
            const double dz = z - sph[4 * s], dy = y - sph[4 * s + 1], dx = x - sph[4 * s + 2], r = sph[4 * s + 3];
            if (dz * dz + dy * dy + dx * dx <= r * r) v = in;
        }
        out[i] = v;
    }
}

// counter-based generator: splitmix64 of (seed, index)
__host__ __device__ inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ inline double unit(uint64_t h) { return ((h >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

// standard normal white noise (Box-Muller on two counter draws per voxel)
__global__ void noise_kernel(long long total, uint64_t seed, double* __restrict__ g) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const uint64_t base = mix64(seed ^ mix64((uint64_t)i));
        const double u1 = unit(mix64(base)), u2 = unit(mix64(base + 1));
        g[i] = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
    }
}

// periodic convolution along one axis with the normalised taps w[-R..R]
// (axis 0: z, 1: y, 2: x of a [Z][Y][X] volume)
__global__ void conv_axis_kernel(const double* __restrict__ src, double* __restrict__ dst, int Z, int Y, int X, int axis,
                                 const double* __restrict__ w, int R) {
    const long long total = (long long)Z * Y * X;
    const int len = axis == 0 ? Z : axis == 1 ? Y : X;
    const long long stride = axis == 0 ? (long long)Y * X : axis == 1 ? X : 1;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)((i / stride) % len);
        const long long base = i - (long long)c * stride;
        double s = 0.0;
        for (int t = -R; t <= R; t++) {
            int q = (c + t) % len;
            if (q < 0) q += len;
            s += w[t + R] * src[base + (long long)q * stride];
        }
        dst[i] = s;
    }
}

// min and max of the volume (one CTA)
__global__ void __launch_bounds__(1024) minmax_kernel(const double* __restrict__ g, long long total,
                                                      double* __restrict__ mm) {
    __shared__ double lo[1024], hi[1024];
    double a = INFINITY, b = -INFINITY;
    for (long long i = threadIdx.x; i < total; i += blockDim.x) {
        a = fmin(a, g[i]);
        b = fmax(b, g[i]);
    }
    lo[threadIdx.x] = a;
    hi[threadIdx.x] = b;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            lo[threadIdx.x] = fmin(lo[threadIdx.x], lo[threadIdx.x + s]);
            hi[threadIdx.x] = fmax(hi[threadIdx.x], hi[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        mm[0] = lo[0];
        mm[1] = hi[0];
    }
}

// n = n_lo + (n_hi - n_lo) t, t = (g - min) / (max - min); kappa t as the imaginary part
__global__ void grf_map_kernel(const double* __restrict__ g, long long total, const double* __restrict__ mm, double n_lo,
                               double n_hi, double kappa, double2* __restrict__ out) {
    const double range = fmax(mm[1] - mm[0], 1e-30);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const double t = (g[i] - mm[0]) / range;
        out[i] = make_double2(n_lo + (n_hi - n_lo) * t, kappa * t);
    }
}

}  // namespace

extern "C" {

scw_status scw_gen_spheres(scw_ctx ctx, int Z, int Y, int X, int n_spheres, const double* spheres,
                           const double* n_background, const double* n_sphere, void* out) {
    if (!ctx || Z < 1 || Y < 1 || X < 1 || n_spheres < 0 || (n_spheres > 0 && !spheres) || !n_background ||
        !n_sphere || !out)
        return fail(SCW_ERR_ARG, "scw_gen_spheres: bad arguments");
    SCW_ON_DEVICE(ctx->device);
    double* d = nullptr;
    SCW_CUDA_TRY(cudaMallocAsync(&d, sizeof(double) * 4 * (size_t)(n_spheres + 1), ctx->stream));
    if (n_spheres > 0)
        SCW_CUDA_TRY(cudaMemcpyAsync(d, spheres, sizeof(double) * 4 * n_spheres, cudaMemcpyHostToDevice, ctx->stream));
    const long long total = (long long)Z * Y * X;
    spheres_kernel<<<std::min<unsigned>(nblk(total), 65535u), 256, 0, ctx->stream>>>(
        Z, Y, X, n_spheres, d, make_double2(n_background[0], n_background[1]), make_double2(n_sphere[0], n_sphere[1]),
        (double2*)out);
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(d, ctx->stream);
    if (e != cudaSuccess) return fail(SCW_ERR_CUDA, cudaGetErrorString(e));
    ctx->launches++;
    SCW_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SCW_OK;
}

scw_status scw_gen_grf(scw_ctx ctx, int Z, int Y, int X, double corr_px, double n_lo, double n_hi, double kappa_max,
                       uint64_t seed, void* out) {
    if (!ctx || Z < 1 || Y < 1 || X < 1 || !(corr_px > 0.0) || !out)
        return fail(SCW_ERR_ARG, "scw_gen_grf: bad arguments");
    SCW_ON_DEVICE(ctx->device);
    const long long total = (long long)Z * Y * X;
    const int R = (int)std::ceil(4.0 * corr_px);
    std::vector<double> w(2 * R + 1);
    double sw = 0.0;
    for (int t = -R; t <= R; t++) sw += (w[t + R] = std::exp(-0.5 * (double)t * t / (corr_px * corr_px)));
    for (double& v : w) v /= sw;
    double *a = nullptr, *b = nullptr, *dw = nullptr;
    cudaStream_t st = ctx->stream;
    if (cudaMallocAsync(&a, sizeof(double) * total, st) != cudaSuccess ||
        cudaMallocAsync(&b, sizeof(double) * total, st) != cudaSuccess ||
        cudaMallocAsync(&dw, sizeof(double) * (w.size() + 2), st) != cudaSuccess) {
        cudaGetLastError();
        if (a) cudaFreeAsync(a, st);
        if (b) cudaFreeAsync(b, st);
        return fail(SCW_ERR_NOMEM, "scw_gen_grf: work buffers");
    }
    const unsigned g = std::min<unsigned>(nblk(total), 65535u);
    cudaMemcpyAsync(dw, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice, st);
    noise_kernel<<<g, 256, 0, st>>>(total, seed, a);
    conv_axis_kernel<<<g, 256, 0, st>>>(a, b, Z, Y, X, 2, dw, R);
    conv_axis_kernel<<<g, 256, 0, st>>>(b, a, Z, Y, X, 1, dw, R);
    conv_axis_kernel<<<g, 256, 0, st>>>(a, b, Z, Y, X, 0, dw, R);
    double* mm = dw + w.size();
    minmax_kernel<<<1, 1024, 0, st>>>(b, total, mm);
    const double kappa = kappa_max * unit(mix64(mix64(seed) ^ 0x6B617070615F3031ull));
    grf_map_kernel<<<g, 256, 0, st>>>(b, total, mm, n_lo, n_hi, kappa, (double2*)out);
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(a, st);
    cudaFreeAsync(b, st);
    cudaFreeAsync(dw, st);
    if (e != cudaSuccess) return fail(SCW_ERR_CUDA, cudaGetErrorString(e));
    ctx->launches += 6;
    SCW_CUDA_TRY(cudaStreamSynchronize(st));
    return SCW_OK;
}

// .npy reader (format 1.0 / 2.0 / 3.0 headers; complex128 '<c16' or float64 '<f8' promoted to
// complex; C or Fortran order; 2-D [Y, X] or 3-D [Z, Y, X]).  dims[3] receives Z, Y, X; with
// out != NULL the volume is streamed in C order into that device buffer (Z Y X complex128)
// through a pinned chunk.  A Fortran-ordered file is transposed on the host chunk by chunk
// only for 2-D; a 3-D Fortran-ordered file is refused (SCW_ERR_UNSUPPORTED).
scw_status scw_npy_read(scw_ctx ctx, const char* path, int* dims, void* out) {
    if (!path || !dims) return fail(SCW_ERR_ARG, "scw_npy_read: null argument");
    FILE* f = fopen(path, "rb");
    if (!f) return fail(SCW_ERR_IO, std::string("cannot open ") + path);
    struct Closer {
        FILE* f;
        ~Closer() { fclose(f); }
    } closer{f};
    unsigned char pre[10];
    if (fread(pre, 1, 10, f) != 10 || std::memcmp(pre, "\x93NUMPY", 6) != 0)
        return fail(SCW_ERR_FORMAT, std::string("not a .npy file: ") + path);
    size_t hlen = 0;
    if (pre[6] == 1) {
        hlen = pre[8] | (pre[9] << 8);
    } else {
        unsigned char more[2];
        if (fread(more, 1, 2, f) != 2) return fail(SCW_ERR_FORMAT, "truncated .npy header");
        hlen = (size_t)pre[8] | ((size_t)pre[9] << 8) | ((size_t)more[0] << 16) | ((size_t)more[1] << 24);
    }
    if (hlen > (1u << 20)) return fail(SCW_ERR_FORMAT, ".npy header too long");
    std::string h(hlen, '\0');
    if (fread(&h[0], 1, hlen, f) != hlen) return fail(SCW_ERR_FORMAT, "truncated .npy header");
    const bool c16 = h.find("'<c16'") != std::string::npos, f8 = h.find("'<f8'") != std::string::npos;
    if (!c16 && !f8) return fail(SCW_ERR_UNSUPPORTED, "scw_npy_read: dtype other than <c16 / <f8");
    const bool fortran = h.find("'fortran_order': True") != std::string::npos;
    const size_t sp = h.find("'shape': (");
    if (sp == std::string::npos) return fail(SCW_ERR_FORMAT, ".npy header without shape");
    std::vector<long long> shp;
    const char* q = h.c_str() + sp + 10;
    while (*q && *q != ')') {
        while (*q == ' ' || *q == ',') q++;
        if (*q == ')') break;
        char* end = nullptr;
        const long long v = strtoll(q, &end, 10);
        if (end == q || v < 0) return fail(SCW_ERR_FORMAT, ".npy shape");
        shp.push_back(v);
        q = end;
    }
    if (shp.size() == 2) shp.insert(shp.begin(), 1);
    if (shp.size() != 3 || shp[0] < 1 || shp[1] < 1 || shp[2] < 1 || shp[0] > (1 << 20) || shp[1] > (1 << 20) ||
        shp[2] > (1 << 20))
        return fail(SCW_ERR_UNSUPPORTED, "scw_npy_read: expected a 2-D or 3-D volume");
    if (fortran && shp[0] != 1) return fail(SCW_ERR_UNSUPPORTED, "scw_npy_read: 3-D Fortran-ordered volume");
    dims[0] = (int)shp[0];
    dims[1] = (int)shp[1];
    dims[2] = (int)shp[2];
    if (!out) return SCW_OK;
    if (!ctx) return fail(SCW_ERR_ARG, "scw_npy_read: null context");
    SCW_ON_DEVICE(ctx->device);
    const long long total = shp[0] * shp[1] * shp[2];
    const size_t esz = c16 ? 16 : 8;
    if (fortran) {                                     // 2-D: read whole, transpose on the host
        std::vector<unsigned char> raw(total * esz);
        if (fread(raw.data(), esz, total, f) != (size_t)total) return fail(SCW_ERR_FORMAT, "truncated .npy data");
        std::vector<double2> v(total);
        const long long Y = shp[1], X = shp[2];
        for (long long y = 0; y < Y; y++)
            for (long long x = 0; x < X; x++) {
                const unsigned char* src = raw.data() + (x * Y + y) * esz;
                double re = 0.0, im = 0.0;
                std::memcpy(&re, src, 8);
                if (c16) std::memcpy(&im, src + 8, 8);
                v[y * X + x] = make_double2(re, im);
            }
        SCW_CUDA_TRY(cudaMemcpy(out, v.data(), sizeof(double2) * total, cudaMemcpyHostToDevice));
        return SCW_OK;
    }
    const long long chunk = 1 << 20;
    double2* pin = nullptr;
    SCW_CUDA_TRY(cudaMallocHost(&pin, sizeof(double2) * chunk));
    struct PinFree {
        double2* p;
        ~PinFree() { cudaFreeHost(p); }
    } pf{pin};
    std::vector<double> tmp(f8 ? chunk : 0);
    for (long long o = 0; o < total; o += chunk) {
        const long long cnt = std::min(chunk, total - o);
        if (c16) {
            if (fread(pin, 16, cnt, f) != (size_t)cnt) return fail(SCW_ERR_FORMAT, "truncated .npy data");
        } else {
            if (fread(tmp.data(), 8, cnt, f) != (size_t)cnt) return fail(SCW_ERR_FORMAT, "truncated .npy data");
            for (long long i = 0; i < cnt; i++) pin[i] = make_double2(tmp[i], 0.0);
        }
        SCW_CUDA_TRY(cudaMemcpy((double2*)out + o, pin, sizeof(double2) * cnt, cudaMemcpyHostToDevice));
    }
    return SCW_OK;
}

}  // extern "C"
