// Plain plane-wave summation on sm_103a:  E(r) = sum_w A_w exp(i k_w . (r - r_ref,w))
//
// Replaces the reference kernels evaluate / kernel_xy / kernel_xz / kernel_yz and the
// host functions gpu_initialize / gpu_cw_evaluate (gpuEvaluator.cu:15-165).
//
// Design (GB300-first, not a translation of the reference's one-thread-per-point loop over
// AoS global memory):
//  * Waves live on the device as SoA tables: Re k and Im k (double, 3 x n), the reference
//    plane z_ref (double) and the amplitude at that plane (complex float, 3 x n).
//  * A CTA evaluates a 16 x 32 tile of points (2 points per thread) against a chunk of one
//    region's waves.  Waves are staged through shared memory 256 at a time; while staging,
//    each thread re-bases one wave to the tile centre r_c in FP64:
//        theta_c = Re k . (r_c - r_ref)  reduced mod 2 pi,   A' = A exp(-Im k . (r_c - r_ref))
//    so the per-(point, wave) work is FP32 over the small in-plane offset d = r - r_c only:
//        theta = theta_c + Re k . d,  m = 2^(-Im k log2(e) . d),  E += A' m (cos theta, i sin theta)
//    i.e. 3 MUFU ops (ex2, sin, cos), 7 FP32 ops and 6 packed f32x2 FMAs per point x wave
//    (2 MUFU and 4 FP32 ops when the batch's waves all have real k).
//  * Tiles that see many waves are split over several CTAs (split-K over the wave list);
//    their FP32 partial sums go to a scratch buffer and a second kernel adds them in a
//    fixed order in FP64 (deterministic, run-to-run bitwise identical).
//  * Regions (which waves a point sees) depend on z only and are resolved on the host per
//    tile row with the reference's rule; rows of a tile in different regions become
//    separate work items.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <new>

#include "scw_internal.h"

namespace scw {

constexpr int kTI = 16;          // tile columns
constexpr int kTJ = 32;          // tile rows
constexpr int kThreads = 256;    // 16 x 16 threads, 2 rows each (j and j + 16)
constexpr int kBatch = 256;      // waves staged in shared memory per step
constexpr int kTilePts = kTI * kTJ;

struct PlaneGeom {
    float a0, b0, c;   // start along i (a) and j (b), fixed coordinate c
    float da, db;      // spacings along i and j
    int Ni, Nj;
    int mode;          // 0: (a,b,c) = (x,y,z); 1: (y,z,x); 2: (x,z,y)
    int pad;
    float* out;        // [Nj][Ni][6] floats
};

struct WorkItem {
    int plane;
    int i0, j0;        // tile origin
    int jr0, jr1;      // rows [jr0, jr1) this item covers (one region)
    int slot;          // partial-sum slot, or -1: write the output directly
    int pad;
    long long w0, w1;  // wave range
};

struct ReduceTile {
    int plane, i0, j0;
    int slot0, nslots;
};

struct WaveSoA {
    const double* kre;
    const double* kim;
    const double* zref;
    const float2* amp;
    long long n;
};

// One staged wave, re-based to the tile centre.  The plane's two in-plane axes are A (along
// the tile columns) and B (along the rows); the out-of-plane offset is zero for every point.
// Amplitudes are stored as duplicated pairs so the accumulation runs on packed f32x2 FMAs:
// P_c += (Ar, Ar) * (ur, ui),  Q_c += (Ai, Ai) * (ur, ui);  E_c = (P.x - Q.y, P.y + Q.x).
struct __align__(16) StagedWave {
    float4 a;   // theta_c (rad, in [-pi, pi]), Re k_A, Re k_B, -Im k_A log2e
    float4 x;   // A'x re, A'x re, A'x im, A'x im
    float4 y;   // A'y ...
    float4 z;   // A'z ...
    float4 b;   // -Im k_B log2e, 0, 0, 0
};

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// d = a * b + c on packed float pairs (sm_100+ f32x2 FMA)
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;"
        : "=l"(d)
        : "l"(*reinterpret_cast<unsigned long long*>(&a)), "l"(*reinterpret_cast<unsigned long long*>(&b)),
          "l"(*reinterpret_cast<unsigned long long*>(&c)));
    return *reinterpret_cast<float2*>(&d);
}

__device__ __forceinline__ float2 lo_pair(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi_pair(float4 v) { return make_float2(v.z, v.w); }

// point coordinates in the reference's float arithmetic: start + d * index, each operation
// rounded separately (no fused multiply-add).
__device__ __forceinline__ float grid_coord(float s, float d, int i) {
    return __fadd_rn(s, __fmul_rn(d, (float)i));
}

__device__ __forceinline__ void to_xyz(int mode, float a, float b, float c, float& x, float& y, float& z) {
    if (mode == 0) { x = a; y = b; z = c; }
    else if (mode == 1) { x = c; y = a; z = b; }
    else { x = a; y = c; z = b; }
}

struct PointAcc {
    float2 p[3], q[3];
};

template <bool kComplexK>
__device__ __forceinline__ void accumulate_point(const StagedWave& w, float kiB, float dA, float dB, PointAcc& acc) {
    const float th = fmaf(w.a.z, dB, fmaf(w.a.y, dA, w.a.x));
    float sn, cs;
    __sincosf(th, &sn, &cs);
    float2 u = make_float2(cs, sn);
    if (kComplexK) {
        const float m = ex2_approx(fmaf(kiB, dB, w.a.w * dA));
        u.x *= m;
        u.y *= m;
    }
    acc.p[0] = ffma2(lo_pair(w.x), u, acc.p[0]);
    acc.q[0] = ffma2(hi_pair(w.x), u, acc.q[0]);
    acc.p[1] = ffma2(lo_pair(w.y), u, acc.p[1]);
    acc.q[1] = ffma2(hi_pair(w.y), u, acc.q[1]);
    acc.p[2] = ffma2(lo_pair(w.z), u, acc.p[2]);
    acc.q[2] = ffma2(hi_pair(w.z), u, acc.q[2]);
}

template <bool kComplexK>
__device__ __forceinline__ void accumulate_batch(const StagedWave* __restrict__ s, int nw, float dA, float dB0,
                                                 float dB1, PointAcc& a0, PointAcc& a1) {
#pragma unroll 2
    for (int k = 0; k < nw; k++) {
        StagedWave w;
        w.a = s[k].a;
        w.x = s[k].x;
        w.y = s[k].y;
        w.z = s[k].z;
        const float kiB = kComplexK ? s[k].b.x : 0.f;
        accumulate_point<kComplexK>(w, kiB, dA, dB0, a0);
        accumulate_point<kComplexK>(w, kiB, dA, dB1, a1);
    }
}

__global__ void __launch_bounds__(kThreads, 4)
plain_eval_kernel(const PlaneGeom* __restrict__ planes, const WorkItem* __restrict__ items, WaveSoA W,
                  float* __restrict__ partials) {
    __shared__ StagedWave sw[kBatch];
    __shared__ double tot[12][kThreads];   // per-thread FP64 running sums (point 0: 0-5, point 1: 6-11)
    const WorkItem it = items[blockIdx.x];
    const PlaneGeom g = planes[it.plane];
    const int t = threadIdx.x;
    const int li = t & 15;
    const int lj = t >> 4;
    const int i = it.i0 + li;
    const int j0 = it.j0 + lj;
    const int j1 = j0 + 16;

    // tile centre: float grid coordinates of tile point (8, 16); per-point in-plane offsets
    const float ac = grid_coord(g.a0, g.da, it.i0 + 8), bc = grid_coord(g.b0, g.db, it.j0 + 16);
    const float dA = (float)((double)grid_coord(g.a0, g.da, i) - (double)ac);
    const float dB0 = (float)((double)grid_coord(g.b0, g.db, j0) - (double)bc);
    const float dB1 = (float)((double)grid_coord(g.b0, g.db, j1) - (double)bc);
    float xc, yc, zc;
    to_xyz(g.mode, ac, bc, g.c, xc, yc, zc);
    // which k components lie along the plane's A and B axes
    const int cA = (g.mode == 1) ? 1 : 0;
    const int cB = (g.mode == 0) ? 1 : 2;

#pragma unroll
    for (int c = 0; c < 12; c++) tot[c][t] = 0.0;
    const double two_pi_hi = 6.283185307179586232;
    const double two_pi_lo = 2.4492935982947064e-16;
    const double inv_two_pi = 0.15915494309189533577;
    const float log2e = 1.44269504088896341f;

    for (long long wb = it.w0; wb < it.w1; wb += kBatch) {
        const int nw = (int)min((long long)kBatch, it.w1 - wb);
        int cplx = 0;
        if (t < nw) {
            const long long w = wb + t;
            const long long n = W.n;
            const double krx = W.kre[w], kry = W.kre[n + w], krz = W.kre[2 * n + w];
            const double kix = W.kim[w], kiy = W.kim[n + w], kiz = W.kim[2 * n + w];
            const double rx = (double)xc, ry = (double)yc, rz = (double)zc - W.zref[w];
            double th = fma(krz, rz, fma(kry, ry, krx * rx));
            const double q = rint(th * inv_two_pi);
            th = fma(-q, two_pi_lo, fma(-q, two_pi_hi, th));
            const double ach = -fma(kiz, rz, fma(kiy, ry, kix * rx));
            const float m = exp2f((float)(ach * 1.4426950408889634074));
            const float2 ax = W.amp[w], ay = W.amp[n + w], az = W.amp[2 * n + w];
            const double krA = cA == 0 ? krx : kry, krB = cB == 1 ? kry : krz;
            const double kiA = cA == 0 ? kix : kiy, kiB = cB == 1 ? kiy : kiz;
            StagedWave s;
            s.a = make_float4((float)th, (float)krA, (float)krB, -(float)kiA * log2e);
            s.x = make_float4(ax.x * m, ax.x * m, ax.y * m, ax.y * m);
            s.y = make_float4(ay.x * m, ay.x * m, ay.y * m, ay.y * m);
            s.z = make_float4(az.x * m, az.x * m, az.y * m, az.y * m);
            s.b = make_float4(-(float)kiB * log2e, 0.f, 0.f, 0.f);
            sw[t] = s;
            cplx = (kiA != 0.0) | (kiB != 0.0);
        }
        cplx = __syncthreads_or(cplx);
        PointAcc a0, a1;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            a0.p[c] = a0.q[c] = a1.p[c] = a1.q[c] = make_float2(0.f, 0.f);
        }
        if (cplx)
            accumulate_batch<true>(sw, nw, dA, dB0, dB1, a0, a1);
        else
            accumulate_batch<false>(sw, nw, dA, dB0, dB1, a0, a1);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            tot[2 * c][t] += (double)(a0.p[c].x - a0.q[c].y);
            tot[2 * c + 1][t] += (double)(a0.p[c].y + a0.q[c].x);
            tot[6 + 2 * c][t] += (double)(a1.p[c].x - a1.q[c].y);
            tot[7 + 2 * c][t] += (double)(a1.p[c].y + a1.q[c].x);
        }
        __syncthreads();
    }

    // rows outside this item's region range contribute zero
    const bool in0 = (j0 >= it.jr0) && (j0 < it.jr1);
    const bool in1 = (j1 >= it.jr0) && (j1 < it.jr1);
    if (it.slot < 0) {
        if (i < g.Ni) {
            if (j0 < g.Nj && in0) {
                float* o = g.out + 6 * ((long long)j0 * g.Ni + i);
#pragma unroll
                for (int c = 0; c < 6; c++) o[c] = (float)tot[c][t];
            }
            if (j1 < g.Nj && in1) {
                float* o = g.out + 6 * ((long long)j1 * g.Ni + i);
#pragma unroll
                for (int c = 0; c < 6; c++) o[c] = (float)tot[6 + c][t];
            }
        }
    } else {
        float* p = partials + (long long)it.slot * kTilePts * 6;
        float* p0 = p + 6 * (lj * kTI + li);
        float* p1 = p + 6 * ((lj + 16) * kTI + li);
#pragma unroll
        for (int c = 0; c < 6; c++) {
            p0[c] = in0 ? (float)tot[c][t] : 0.f;
            p1[c] = in1 ? (float)tot[6 + c][t] : 0.f;
        }
    }
}

__global__ void __launch_bounds__(kThreads)
plain_reduce_kernel(const PlaneGeom* __restrict__ planes, const ReduceTile* __restrict__ tiles,
                    const float* __restrict__ partials) {
    const ReduceTile rt = tiles[blockIdx.x];
    const PlaneGeom g = planes[rt.plane];
    for (int q = threadIdx.x; q < kTilePts; q += blockDim.x) {
        const int li = q % kTI, lj = q / kTI;
        const int i = rt.i0 + li, j = rt.j0 + lj;
        double s[6] = {0, 0, 0, 0, 0, 0};
        for (int k = 0; k < rt.nslots; k++) {
            const float* p = partials + ((long long)(rt.slot0 + k) * kTilePts + q) * 6;
#pragma unroll
            for (int c = 0; c < 6; c++) s[c] += (double)p[c];
        }
        if (i < g.Ni && j < g.Nj) {
            float* o = g.out + 6 * ((long long)j * g.Ni + i);
#pragma unroll
            for (int c = 0; c < 6; c++) o[c] = (float)s[c];
        }
    }
}

// ------------------------------------------------------------------------------------
// Host planning
// ------------------------------------------------------------------------------------
static inline float host_grid_coord(float s, float d, int i) {
    volatile float p = d * (float)i;   // rounded product, then rounded sum (no contraction)
    volatile float r = s + p;
    return r;
}

static int64_t region_of(const scw_waves_s* w, float z) {
    // gpuEvaluator.cu:31-37 (rule 0) / cpuEvaluator.cpp:300-305 (rule 1): last satisfied wins
    int64_t l = 0;
    const double zd = (double)z;
    for (int li = 0; li < w->layers; li++) {
        const double thr = (w->rule == 0) ? (double)w->z_layers[li] - 0.001 : (double)w->z_layers[li];
        if (zd >= thr) l = li + 1;
    }
    return l;
}

struct Plan {
    std::vector<WorkItem> items;
    std::vector<ReduceTile> rtiles;
    int nslots = 0;
};

static void plan_planes(const scw_waves_s* w, const std::vector<PlaneGeom>& planes, int sm_count, Plan& P) {
    // total work to choose the split-K chunk: aim for >= 6 CTAs per SM when there is enough
    long long tiles = 0;
    double work = 0;
    for (const auto& g : planes) {
        long long nt = (long long)((g.Ni + kTI - 1) / kTI) * ((g.Nj + kTJ - 1) / kTJ);
        tiles += nt;
        if (g.mode == 0) {
            int64_t r = region_of(w, g.c);
            work += (double)nt * (double)(w->end[r] - w->begin[r]);
        } else {
            for (int j = 0; j < g.Nj; j++) {
                int64_t r = region_of(w, host_grid_coord(g.b0, g.db, j));
                work += (double)((g.Ni + kTI - 1) / kTI) * (double)(w->end[r] - w->begin[r]) / kTJ;
            }
        }
    }
    const double target_items = 48.0 * sm_count;
    long long chunk = (long long)std::ceil(work / std::max(1.0, target_items));
    chunk = std::max<long long>(chunk, 4 * kBatch);
    chunk = ((chunk + kBatch - 1) / kBatch) * kBatch;

    std::vector<int64_t> row_region;
    for (int pi = 0; pi < (int)planes.size(); pi++) {
        const auto& g = planes[pi];
        row_region.assign(g.Nj, 0);
        if (g.mode == 0) {
            std::fill(row_region.begin(), row_region.end(), region_of(w, g.c));
        } else {
            for (int j = 0; j < g.Nj; j++) row_region[j] = region_of(w, host_grid_coord(g.b0, g.db, j));
        }
        for (int j0 = 0; j0 < g.Nj; j0 += kTJ) {
            const int jend = std::min(g.Nj, j0 + kTJ);
            for (int i0 = 0; i0 < g.Ni; i0 += kTI) {
                // group rows of the tile by region
                std::vector<WorkItem> tile_items;
                int jr = j0;
                while (jr < jend) {
                    int je = jr + 1;
                    while (je < jend && row_region[je] == row_region[jr]) je++;
                    const int64_t r = row_region[jr];
                    const long long b = w->begin[r], e = w->end[r];
                    for (long long c0 = b; c0 < e; c0 += chunk) {
                        WorkItem it{};
                        it.plane = pi;
                        it.i0 = i0;
                        it.j0 = j0;
                        it.jr0 = jr;
                        it.jr1 = je;
                        it.w0 = c0;
                        it.w1 = std::min(e, c0 + chunk);
                        tile_items.push_back(it);
                    }
                    jr = je;
                }
                if (tile_items.empty()) {   // no waves anywhere in the tile: write zeros
                    WorkItem it{};
                    it.plane = pi;
                    it.i0 = i0;
                    it.j0 = j0;
                    it.jr0 = j0;
                    it.jr1 = jend;
                    it.w0 = it.w1 = 0;
                    tile_items.push_back(it);
                }
                if (tile_items.size() == 1 && tile_items[0].jr0 == j0 && tile_items[0].jr1 == jend) {
                    tile_items[0].slot = -1;
                    P.items.push_back(tile_items[0]);
                } else {
                    ReduceTile rt{pi, i0, j0, P.nslots, (int)tile_items.size()};
                    for (auto& it : tile_items) {
                        it.slot = P.nslots++;
                        P.items.push_back(it);
                    }
                    P.rtiles.push_back(rt);
                }
            }
        }
    }
}

static scw_status launch_planes(scw_waves w, std::vector<PlaneGeom>& planes) {
    scw_ctx ctx = w->ctx;
    SCW_ON_DEVICE(ctx->device);
    Plan P;
    plan_planes(w, planes, ctx->sm_count, P);
    if (P.items.empty()) return SCW_OK;
    // longest items first, so the short exterior-region items fill the tail of the grid
    std::stable_sort(P.items.begin(), P.items.end(),
                     [](const WorkItem& a, const WorkItem& b) { return (a.w1 - a.w0) > (b.w1 - b.w0); });

    const size_t planes_bytes = planes.size() * sizeof(PlaneGeom);
    const size_t items_off = (planes_bytes + 255) / 256 * 256;
    const size_t items_bytes = P.items.size() * sizeof(WorkItem);
    const size_t rt_off = (items_off + items_bytes + 255) / 256 * 256;
    const size_t rt_bytes = P.rtiles.size() * sizeof(ReduceTile);
    const size_t total = rt_off + rt_bytes;

    // the pinned staging buffer may still be read by the previous upload
    SCW_CUDA_TRY(cudaEventSynchronize(ctx->desc_done));
    scw_status st = ctx->host_desc.reserve(total);
    if (st != SCW_OK) return st;
    st = ctx->desc.reserve(total);
    if (st != SCW_OK) return st;
    char* h = (char*)ctx->host_desc.ptr;
    std::memcpy(h, planes.data(), planes_bytes);
    std::memcpy(h + items_off, P.items.data(), items_bytes);
    if (rt_bytes) std::memcpy(h + rt_off, P.rtiles.data(), rt_bytes);
    SCW_CUDA_TRY(cudaMemcpyAsync(ctx->desc.ptr, h, total, cudaMemcpyHostToDevice, ctx->stream));
    SCW_CUDA_TRY(cudaEventRecord(ctx->desc_done, ctx->stream));
    if (P.nslots) {
        st = ctx->scratch.reserve((size_t)P.nslots * kTilePts * 6 * sizeof(float));
        if (st != SCW_OK) return st;
    }
    char* d = (char*)ctx->desc.ptr;
    const PlaneGeom* dplanes = (const PlaneGeom*)d;
    const WorkItem* ditems = (const WorkItem*)(d + items_off);
    const ReduceTile* drt = (const ReduceTile*)(d + rt_off);
    WaveSoA soa{w->kre, w->kim, w->zref, w->amp, (long long)w->n};
    {
        LaunchTimer lt(ctx, "plain_eval_kernel");
        plain_eval_kernel<<<(unsigned)P.items.size(), kThreads, 0, ctx->stream>>>(dplanes, ditems, soa,
                                                                                (float*)ctx->scratch.ptr);
    }
    SCW_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    if (!P.rtiles.empty()) {
        LaunchTimer lt(ctx, "plain_reduce_kernel");
        plain_reduce_kernel<<<(unsigned)P.rtiles.size(), kThreads, 0, ctx->stream>>>(dplanes, drt,
                                                                                   (const float*)ctx->scratch.ptr);
        SCW_CUDA_TRY(cudaGetLastError());
        ctx->launches++;
    }
    return SCW_OK;
}

scw_status waves_upload(scw_waves w, const std::vector<double>& kre, const std::vector<double>& kim,
                        const std::vector<double>& zref, const std::vector<float2>& amp) {
    scw_ctx ctx = w->ctx;
    SCW_ON_DEVICE(ctx->device);
    const size_t n = (size_t)w->n;
    if (n == 0) return SCW_OK;
    if (cudaMalloc(&w->kre, 3 * n * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&w->kim, 3 * n * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&w->zref, n * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&w->amp, 3 * n * sizeof(float2)) != cudaSuccess)
        return fail(SCW_ERR_NOMEM, "cudaMalloc of the wave tables");
    SCW_CUDA_TRY(cudaMemcpyAsync(w->kre, kre.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    SCW_CUDA_TRY(cudaMemcpyAsync(w->kim, kim.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    SCW_CUDA_TRY(cudaMemcpyAsync(w->zref, zref.data(), n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    SCW_CUDA_TRY(cudaMemcpyAsync(w->amp, amp.data(), 3 * n * sizeof(float2), cudaMemcpyHostToDevice, ctx->stream));
    SCW_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SCW_OK;
}

}  // namespace scw

using scw::fail;

static void free_waves(scw_waves w) {
    if (!w) return;
    ::scw::DeviceScope dev_scope_(w->ctx ? w->ctx->device : -1);
    if (w->kre) cudaFree(w->kre);
    if (w->kim) cudaFree(w->kim);
    if (w->zref) cudaFree(w->zref);
    if (w->amp) cudaFree(w->amp);
    delete w;
}

extern "C" {

scw_status scw_gpu_initialize(scw_ctx ctx, int layers, const float* z_layers, const int* waves_begin,
                              const int* waves_end, const float* W, int64_t n_waves, scw_waves* out) {
    if (!ctx || !out || layers < 0 || n_waves < 0 || !waves_begin || !waves_end || (layers && !z_layers) ||
        (n_waves && !W))
        return fail(SCW_ERR_ARG, "scw_gpu_initialize: bad arguments");
    *out = nullptr;
    for (int l = 0; l <= layers; l++) {
        if (waves_begin[l] < 0 || waves_end[l] < waves_begin[l] || waves_end[l] > n_waves)
            return fail(SCW_ERR_ARG, "scw_gpu_initialize: region " + std::to_string(l) + " outside the wave table");
    }
    scw_waves w = new (std::nothrow) scw_waves_s();
    if (!w) return fail(SCW_ERR_NOMEM, "host allocation");
    w->ctx = ctx;
    w->layers = layers;
    w->n = n_waves;
    w->z_layers.assign(z_layers, z_layers + layers);
    w->begin.assign(waves_begin, waves_begin + layers + 1);
    w->end.assign(waves_end, waves_end + layers + 1);
    const size_t n = (size_t)n_waves;
    std::vector<double> kre(3 * n), kim(3 * n), zref(n, 0.0);
    std::vector<float2> amp(3 * n);
    for (size_t i = 0; i < n; i++) {
        const float* r = W + 12 * i;
        for (int c = 0; c < 3; c++) {
            amp[c * n + i] = make_float2(r[2 * c], r[2 * c + 1]);
            kre[c * n + i] = (double)r[6 + 2 * c];
            kim[c * n + i] = (double)r[7 + 2 * c];
        }
    }
    scw_status st = scw::waves_upload(w, kre, kim, zref, amp);
    if (st != SCW_OK) {
        free_waves(w);
        return st;
    }
    *out = w;
    return SCW_OK;
}

scw_status scw_gpu_initialize_cw(scw_ctx ctx, scw_cw cw, scw_waves* out) {
    if (!ctx || !cw || !out) return fail(SCW_ERR_ARG, "scw_gpu_initialize_cw: null argument");
    *out = nullptr;
    int layers = 0;
    int64_t total = 0;
    scw_status st = scw_cw_allocate(cw, &layers, &total);
    if (st != SCW_OK) return st;
    scw_waves w = new (std::nothrow) scw_waves_s();
    if (!w) return fail(SCW_ERR_NOMEM, "host allocation");
    w->ctx = ctx;
    w->layers = layers;
    w->n = total;
    const size_t n = (size_t)total;
    std::vector<double> kre(3 * n), kim(3 * n), zref(n);
    std::vector<float2> amp(3 * n);
    size_t idx = 0;
    // Re-reference each wave of layer l from the origin to z_l in FP64:
    // E0_cw exp(i k.r) = (E0_cw exp(i kz z_l)) exp(i k.(r - (0,0,z_l))).
    auto add = [&](const std::vector<double>& src, double zl) {
        const size_t m = src.size() / 12;
        for (size_t q = 0; q < m; q++, idx++) {
            const double* r = src.data() + 12 * q;
            const std::complex<double> kz(r[10], r[11]);
            const std::complex<double> f = std::exp(std::complex<double>(0.0, 1.0) * kz * zl);
            for (int c = 0; c < 3; c++) {
                std::complex<double> e(r[2 * c], r[2 * c + 1]);
                e *= f;
                amp[c * n + idx] = make_float2((float)e.real(), (float)e.imag());
                kre[c * n + idx] = r[6 + 2 * c];
                kim[c * n + idx] = r[7 + 2 * c];
            }
            zref[idx] = zl;
        }
    };
    w->begin.assign(layers + 1, 0);
    w->end.assign(layers + 1, 0);
    w->z_layers.resize(layers);
    add(cw->Pi, 0.0);
    for (int l = 0; l < layers; l++) {
        const auto& L = cw->layers[(size_t)l];
        w->z_layers[l] = (float)L.z;
        add(L.Pr, L.z);
        w->end[l] = (int64_t)idx;
        w->begin[l + 1] = (int64_t)idx;
        add(L.Pt, L.z);
    }
    w->end[layers] = (int64_t)idx;
    st = scw::waves_upload(w, kre, kim, zref, amp);
    if (st != SCW_OK) {
        free_waves(w);
        return st;
    }
    *out = w;
    return SCW_OK;
}

scw_status scw_waves_destroy(scw_waves w) {
    free_waves(w);
    return SCW_OK;
}

scw_status scw_waves_set_region_rule(scw_waves w, int rule) {
    if (!w || (rule != 0 && rule != 1)) return fail(SCW_ERR_ARG, "region rule must be 0 or 1");
    w->rule = rule;
    return SCW_OK;
}

scw_status scw_waves_info(scw_waves w, int* layers, int64_t* n_waves) {
    if (!w) return fail(SCW_ERR_ARG, "null wave set");
    if (layers) *layers = w->layers;
    if (n_waves) *n_waves = w->n;
    return SCW_OK;
}

static scw::PlaneGeom make_plane(int mode, float a0, float b0, float c, float da, float db, int Ni, int Nj,
                                 float* out) {
    scw::PlaneGeom g{};
    g.a0 = a0;
    g.b0 = b0;
    g.c = c;
    g.da = da;
    g.db = db;
    g.Ni = Ni;
    g.Nj = Nj;
    g.mode = mode;
    g.out = out;
    return g;
}

scw_status scw_eval_plane_device(scw_waves w, int axis, float a_start, float b_start, float c, float d, int N,
                                 float* dE) {
    if (!w || !dE || N <= 0 || axis < 0 || axis > 2) return fail(SCW_ERR_ARG, "scw_eval_plane_device: bad arguments");
    std::vector<scw::PlaneGeom> planes{make_plane(axis, a_start, b_start, c, d, d, N, N, dE)};
    return scw::launch_planes(w, planes);
}

scw_status scw_eval_volume_device(scw_waves w, float x_start, float y_start, float z_start, float dx, float dy,
                                  float dz, int Nx, int Ny, int Nz, float* dE) {
    if (!w || !dE || Nx <= 0 || Ny <= 0 || Nz <= 0) return fail(SCW_ERR_ARG, "scw_eval_volume_device: bad arguments");
    std::vector<scw::PlaneGeom> planes;
    planes.reserve(Nz);
    for (int k = 0; k < Nz; k++) {
        const float z = scw::host_grid_coord(z_start, dz, k);
        planes.push_back(make_plane(0, x_start, y_start, z, dx, dy, Nx, Ny, dE + (size_t)k * Nx * Ny * 6));
    }
    return scw::launch_planes(w, planes);
}

// gpu_cw_evaluate (gpuEvaluator.cu:131-165): xy plane at z, xz plane at y, yz plane at x;
// the three planes run in one launch and come back to the caller's host arrays.
scw_status scw_gpu_cw_evaluate(scw_waves w, float* E_xy, float* E_xz, float* E_yz, float x_start, float y_start,
                               float z_start, float x, float y, float z, float d, int N, int device) {
    if (!w || !E_xy || !E_xz || !E_yz || N <= 0) return fail(SCW_ERR_ARG, "scw_gpu_cw_evaluate: bad arguments");
    scw_ctx ctx = w->ctx;
    if (device != ctx->device)
        return fail(SCW_ERR_ARG, "scw_gpu_cw_evaluate: device differs from the wave set's device");
    SCW_ON_DEVICE(ctx->device);
    const size_t plane_floats = (size_t)N * N * 6;
    scw_status st = ctx->planes_out.reserve(3 * plane_floats * sizeof(float));
    if (st != SCW_OK) return st;
    float* dxy = (float*)ctx->planes_out.ptr;
    float* dxz = dxy + plane_floats;
    float* dyz = dxz + plane_floats;
    std::vector<scw::PlaneGeom> planes{make_plane(0, x_start, y_start, z, d, d, N, N, dxy),
                                       make_plane(2, x_start, z_start, y, d, d, N, N, dxz),
                                       make_plane(1, y_start, z_start, x, d, d, N, N, dyz)};
    st = scw::launch_planes(w, planes);
    if (st != SCW_OK) return st;
    SCW_CUDA_TRY(cudaMemcpyAsync(E_xy, dxy, plane_floats * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    SCW_CUDA_TRY(cudaMemcpyAsync(E_xz, dxz, plane_floats * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    SCW_CUDA_TRY(cudaMemcpyAsync(E_yz, dyz, plane_floats * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    SCW_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SCW_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------
// Allocation-free plane evaluation
//
// For callers that must not allocate GPU memory while they run: a host application that
// sub-allocates one pre-sized pool for everything and treats any other cudaMalloc as a
// leak, a real-time viewer that may not stall on the allocator in its frame loop, or a
// plug-in host that forbids its plug-ins from allocating device memory.  The entry point
// below evaluates one plane like scw_eval_plane_device but takes its split-K scratch from
// a fixed array compiled into this library, passes its tiny descriptor tables as kernel
// parameters, and calls no cudaMalloc, cudaMallocHost, cudaFree or allocating library
// routine.
// ------------------------------------------------------------------------------------

namespace scw {

constexpr int kStaticMaxLayers = 160;   // layer thresholds carried as kernel parameters
constexpr int kStaticMaxN = 16384;      // plane edge
constexpr int kStaticMaxSplit = 64;
constexpr int kStaticSlots = 1024;      // partial-sum tiles held by the scratch array
constexpr size_t kStaticScratchFloats = (size_t)kStaticSlots * kTilePts * 6;   // 12 MiB

// Split-K partial sums of the allocation-free path.  Every GPU that loads this library holds
// this array until the process exits.  Host code must not use its name as a pointer: on the
// host it is only a stand-in for the symbol, and its device address comes from
// cudaGetSymbolAddress (static_scratch below).
static __device__ __align__(256) float g_static_partials[kStaticScratchFloats];

struct StaticRegions {
    long long begin[kStaticMaxLayers + 1];
    long long end[kStaticMaxLayers + 1];
    float z[kStaticMaxLayers];
    int layers;
    int rule;
};

__device__ __forceinline__ int static_region_of(const StaticRegions& R, float z) {
    // same rule as region_of on the host: the last satisfied threshold wins
    int l = 0;
    const double zd = (double)z;
    for (int li = 0; li < R.layers; li++) {
        const double thr = (R.rule == 0) ? (double)R.z[li] - 0.001 : (double)R.z[li];
        if (zd >= thr) l = li + 1;
    }
    return l;
}

// One CTA = one 16 x 32 tile and one of `split` parts of the wave list of every region its
// rows fall in.  split == 1: the CTA writes the output; otherwise partial slot
// (tile * split + part) of `partials`, every float of it, so nothing has to start at zero.
__global__ void __launch_bounds__(kThreads, 4)
plain_eval_static_kernel(const __grid_constant__ StaticRegions R, PlaneGeom g, int tiles_i, int split, WaveSoA W,
                         float* __restrict__ partials) {
    __shared__ StagedWave sw[kBatch];
    __shared__ double tot[12][kThreads];
    __shared__ int row_region[kTJ];
    const int tile = blockIdx.x;
    const int part = blockIdx.y;
    const int ti0 = (tile % tiles_i) * kTI, tj0 = (tile / tiles_i) * kTJ;
    const int t = threadIdx.x;
    const int li = t & 15;
    const int lj = t >> 4;
    const int i = ti0 + li;
    const int j0 = tj0 + lj;
    const int j1 = j0 + 16;

    const float ac = grid_coord(g.a0, g.da, ti0 + 8), bc = grid_coord(g.b0, g.db, tj0 + 16);
    const float dA = (float)((double)grid_coord(g.a0, g.da, i) - (double)ac);
    const float dB0 = (float)((double)grid_coord(g.b0, g.db, j0) - (double)bc);
    const float dB1 = (float)((double)grid_coord(g.b0, g.db, j1) - (double)bc);
    float xc, yc, zc;
    to_xyz(g.mode, ac, bc, g.c, xc, yc, zc);
    const int cA = (g.mode == 1) ? 1 : 0;
    const int cB = (g.mode == 0) ? 1 : 2;

    if (t < kTJ) {
        const int j = tj0 + t;
        row_region[t] = (j < g.Nj) ? static_region_of(R, g.mode == 0 ? g.c : grid_coord(g.b0, g.db, j)) : -1;
    }
#pragma unroll
    for (int c = 0; c < 12; c++) tot[c][t] = 0.0;
    __syncthreads();

    const double two_pi_hi = 6.283185307179586232;
    const double two_pi_lo = 2.4492935982947064e-16;
    const double inv_two_pi = 0.15915494309189533577;
    const float log2e = 1.44269504088896341f;

    // runs of consecutive rows in one region; the loop bounds come from shared memory, so
    // every thread of the CTA takes the same path
    int row = 0;
    while (row < kTJ && row_region[row] >= 0) {
        const int r = row_region[row];
        int re = row + 1;
        while (re < kTJ && row_region[re] == r) re++;
        const bool in0 = lj >= row && lj < re;
        const bool in1 = lj + 16 >= row && lj + 16 < re;
        const long long b = R.begin[r], e = R.end[r];
        long long chunk = (e - b + split - 1) / split;
        chunk = (chunk + kBatch - 1) / kBatch * kBatch;
        const long long w0 = min(e, b + (long long)part * chunk), w1 = min(e, w0 + chunk);
        for (long long wb = w0; wb < w1; wb += kBatch) {
            const int nw = (int)min((long long)kBatch, w1 - wb);
            int cplx = 0;
            if (t < nw) {
                const long long w = wb + t;
                const long long n = W.n;
                const double krx = W.kre[w], kry = W.kre[n + w], krz = W.kre[2 * n + w];
                const double kix = W.kim[w], kiy = W.kim[n + w], kiz = W.kim[2 * n + w];
                const double rx = (double)xc, ry = (double)yc, rz = (double)zc - W.zref[w];
                double th = fma(krz, rz, fma(kry, ry, krx * rx));
                const double q = rint(th * inv_two_pi);
                th = fma(-q, two_pi_lo, fma(-q, two_pi_hi, th));
                const double ach = -fma(kiz, rz, fma(kiy, ry, kix * rx));
                const float m = exp2f((float)(ach * 1.4426950408889634074));
                const float2 ax = W.amp[w], ay = W.amp[n + w], az = W.amp[2 * n + w];
                const double krA = cA == 0 ? krx : kry, krB = cB == 1 ? kry : krz;
                const double kiA = cA == 0 ? kix : kiy, kiB = cB == 1 ? kiy : kiz;
                StagedWave s;
                s.a = make_float4((float)th, (float)krA, (float)krB, -(float)kiA * log2e);
                s.x = make_float4(ax.x * m, ax.x * m, ax.y * m, ax.y * m);
                s.y = make_float4(ay.x * m, ay.x * m, ay.y * m, ay.y * m);
                s.z = make_float4(az.x * m, az.x * m, az.y * m, az.y * m);
                s.b = make_float4(-(float)kiB * log2e, 0.f, 0.f, 0.f);
                sw[t] = s;
                cplx = (kiA != 0.0) | (kiB != 0.0);
            }
            cplx = __syncthreads_or(cplx);
            PointAcc a0, a1;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                a0.p[c] = a0.q[c] = a1.p[c] = a1.q[c] = make_float2(0.f, 0.f);
            }
            if (cplx)
                accumulate_batch<true>(sw, nw, dA, dB0, dB1, a0, a1);
            else
                accumulate_batch<false>(sw, nw, dA, dB0, dB1, a0, a1);
            if (in0) {
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    tot[2 * c][t] += (double)(a0.p[c].x - a0.q[c].y);
                    tot[2 * c + 1][t] += (double)(a0.p[c].y + a0.q[c].x);
                }
            }
            if (in1) {
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    tot[6 + 2 * c][t] += (double)(a1.p[c].x - a1.q[c].y);
                    tot[7 + 2 * c][t] += (double)(a1.p[c].y + a1.q[c].x);
                }
            }
            __syncthreads();
        }
        row = re;
    }

    if (split == 1) {
        if (i < g.Ni) {
            if (j0 < g.Nj) {
                float* o = g.out + 6 * ((long long)j0 * g.Ni + i);
#pragma unroll
                for (int c = 0; c < 6; c++) o[c] = (float)tot[c][t];
            }
            if (j1 < g.Nj) {
                float* o = g.out + 6 * ((long long)j1 * g.Ni + i);
#pragma unroll
                for (int c = 0; c < 6; c++) o[c] = (float)tot[6 + c][t];
            }
        }
    } else {
        float* p = partials + ((long long)tile * split + part) * kTilePts * 6;
        float* p0 = p + 6 * (lj * kTI + li);
        float* p1 = p + 6 * ((lj + 16) * kTI + li);
#pragma unroll
        for (int c = 0; c < 6; c++) {
            p0[c] = (float)tot[c][t];
            p1[c] = (float)tot[6 + c][t];
        }
    }
}

// adds the `split` partial slots of each tile in a fixed order, in FP64
__global__ void __launch_bounds__(kThreads)
plain_reduce_static_kernel(PlaneGeom g, int tiles_i, int split, const float* __restrict__ partials) {
    const int tile = blockIdx.x;
    const int ti0 = (tile % tiles_i) * kTI, tj0 = (tile / tiles_i) * kTJ;
    for (int q = threadIdx.x; q < kTilePts; q += blockDim.x) {
        const int i = ti0 + q % kTI, j = tj0 + q / kTI;
        double s[6] = {0, 0, 0, 0, 0, 0};
        for (int k = 0; k < split; k++) {
            const float* p = partials + (((long long)tile * split + k) * kTilePts + q) * 6;
#pragma unroll
            for (int c = 0; c < 6; c++) s[c] += (double)p[c];
        }
        if (i < g.Ni && j < g.Nj) {
            float* o = g.out + 6 * ((long long)j * g.Ni + i);
#pragma unroll
            for (int c = 0; c < 6; c++) o[c] = (float)s[c];
        }
    }
}

// Device address of g_static_partials as seen from the context's device, looked up once per
// context with that device current (the first lookup may load this library's GPU module
// there) and kept in the context.  A context made after a cudaDeviceReset looks it up afresh.
static scw_status static_scratch(scw_ctx ctx, float** out) {
    if (!ctx->static_scratch) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_partials);
        if (e != cudaSuccess || !p)
            return fail(SCW_ERR_CUDA, std::string("cudaGetSymbolAddress of the static scratch array: ") +
                                          cudaGetErrorString(e));
        ctx->static_scratch = p;
    }
    *out = (float*)ctx->static_scratch;
    return SCW_OK;
}

}  // namespace scw

extern "C" {

scw_status scw_eval_plane_device_static(scw_waves w, int axis, float a_start, float b_start, float c, float d, int N,
                                        float* dE) {
    using namespace scw;
    if (!w || !dE || N <= 0 || axis < 0 || axis > 2)
        return fail(SCW_ERR_ARG, "scw_eval_plane_device_static: bad arguments");
    if (N > kStaticMaxN)
        return fail(SCW_ERR_ARG, "scw_eval_plane_device_static: N = " + std::to_string(N) +
                                     " exceeds the maximum plane edge " + std::to_string(kStaticMaxN));
    if (w->layers > kStaticMaxLayers)
        return fail(SCW_ERR_ARG, "scw_eval_plane_device_static: " + std::to_string(w->layers) +
                                     " layers exceed the maximum of " + std::to_string(kStaticMaxLayers));
    scw_ctx ctx = w->ctx;
    SCW_ON_DEVICE(ctx->device);
    float* scratch = nullptr;
    scw_status st = static_scratch(ctx, &scratch);
    if (st != SCW_OK) return st;

    StaticRegions R;
    R.layers = w->layers;
    R.rule = w->rule;
    for (int l = 0; l < kStaticMaxLayers; l++) R.z[l] = l < w->layers ? w->z_layers[l] : 0.f;
    for (int l = 0; l <= kStaticMaxLayers; l++) {
        R.begin[l] = l <= w->layers ? (long long)w->begin[l] : 0;
        R.end[l] = l <= w->layers ? (long long)w->end[l] : 0;
    }
    long long longest = 0;
    for (int l = 0; l <= w->layers; l++) longest = std::max<long long>(longest, w->end[l] - w->begin[l]);

    PlaneGeom g{};
    g.a0 = a_start;
    g.b0 = b_start;
    g.c = c;
    g.da = d;
    g.db = d;
    g.Ni = N;
    g.Nj = N;
    g.mode = axis;
    g.out = dE;
    const int tiles_i = (N + kTI - 1) / kTI, tiles_j = (N + kTJ - 1) / kTJ;
    const int tiles = tiles_i * tiles_j;
    // split the wave lists so about 24 CTAs per SM run, at least 4 batches per part, and the
    // partial sums fit the scratch array (planes of more than kStaticSlots tiles run unsplit)
    int split = (int)std::min<long long>(kStaticMaxSplit, (24LL * ctx->sm_count + tiles - 1) / tiles);
    split = (int)std::min<long long>(split, std::max<long long>(1, (longest + 4 * kBatch - 1) / (4 * kBatch)));
    split = std::min(split, std::max(1, kStaticSlots / tiles));
    split = std::max(split, 1);

    plain_eval_static_kernel<<<dim3((unsigned)tiles, (unsigned)split), kThreads, 0, ctx->stream>>>(
        R, g, tiles_i, split, WaveSoA{w->kre, w->kim, w->zref, w->amp, (long long)w->n}, scratch);
    SCW_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    if (split > 1) {
        plain_reduce_static_kernel<<<(unsigned)tiles, kThreads, 0, ctx->stream>>>(g, tiles_i, split, scratch);
        SCW_CUDA_TRY(cudaGetLastError());
        ctx->launches++;
    }
    return SCW_OK;
}

}  // extern "C"
