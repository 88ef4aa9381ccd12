// Separable ("GEMM form") field evaluation.
//
// Inside slice l the solver's waves share kx, ky per harmonic p = (a, b) of an M0 x M1
// grid and kz per eigenmode j (sCWatter.cpp:904-952), so
//     E_c(x, y, z) = sum_a e^{i kx_a x} sum_b e^{i ky_b y} C_c(a, b; z),
//     C_c(p; z)   = sum_j Qdn_c(p, j) e^{i kzdn_j (z - z_l)} + sum_j Qup_c(p, j) e^{i kzup_j (z - z_{l+1})}.
// Stage 1 (HBM-bound): C for every evaluated z-plane (sep_phase_kernel + sep_contract_kernel;
//   sep_exterior_kernel for the incident/reflected and transmitted regions).
// Stage 2: T_c(row, a) = sum_b e^{i ky_b y_row} C_c(a, b; z_row) (sep_rows_kernel), then the
//   output GEMM E_c(row, x) = sum_a T_c(row, a) e^{i kx_a x}: FP32 SIMT (sep_synth_kernel) or
//   tcgen05 3xTF32 / split-BF16 (eval_sep_tc.cu).
// Phases are reduced in FP64 before rounding to FP32.  The yz plane contracts a first and
// keeps b (ky) as the output axis.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <new>

#include "scw_internal.h"
#include "scw_sep.h"

namespace scw {


// exp(i kz (z - zref)) with the angle reduced in FP64
__device__ __forceinline__ float2 phase_fp64(double kr, double ki, double dz) {
    const double th = kr * dz;
    const double q = rint(th * 0.15915494309189533577);
    const double t = fma(-q, 2.4492935982947064e-16, fma(-q, 6.283185307179586232, th));
    const float m = expf((float)(-ki * dz));
    float s, c;
    sincosf((float)t, &s, &c);
    return make_float2(m * c, m * s);
}

// Phase table of one group of planes, Phi[g][h][j][kk] (h = 0, 1; kk < nks; zero past g.nk):
//   two-half sets: h = 0: exp(i kz_dn_j (z_kk - z_l)), h = 1: exp(i kz_up_j (z_kk - z_{l+1}));
//   paired sets (beta != null): the mode amplitudes folded in, in FP64,
//     h = 0 (rows Ex, Ey): beta_dn_j exp(i kz_dn_j (z - z_l)) + beta_up_j exp(i kz_up_j (z - z_{l+1}))
//     h = 1 (rows Ez):     beta_dn_j exp(i kz_dn_j (z - z_l)) - beta_up_j exp(i kz_up_j (z - z_{l+1}))
__global__ void sep_phase_kernel(const PGroup* __restrict__ groups, const float* __restrict__ zlist,
                                 const double2* __restrict__ kz, const double2* __restrict__ beta,
                                 const double* __restrict__ zb, int J, int nks, float2* __restrict__ Phi) {
    const PGroup g = groups[blockIdx.y];
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int l = g.region - 1;
    if (!beta) {
        // two-half set: one thread per (half, mode), j < 2 J
        if (j >= 2 * J) return;
        const int half = j / J, jj = j - half * J;
        float2* out = Phi + ((long long)blockIdx.y * 2 * J + j) * nks;
        const double2 k = kz[((long long)l * 2 + half) * J + jj];
        const double zref = half == 0 ? zb[l] : zb[l + 1];
        for (int kk = 0; kk < nks; kk++) {
            if (kk < g.nk) {
                const double dz = (double)zlist[g.zi[kk]] - zref;
                out[kk] = phase_fp64(k.x, k.y, dz);
            } else {
                out[kk] = make_float2(0.f, 0.f);
            }
        }
        return;
    }
    // paired set: one thread per mode j < J writes both halves from the same two phases
    if (j >= J) return;
    const int jj = j;
    float2* out0 = Phi + ((long long)blockIdx.y * 2 * J + jj) * nks;
    float2* out1 = Phi + ((long long)blockIdx.y * 2 * J + J + jj) * nks;
    const double2 kd = kz[(long long)l * 2 * J + jj], ku = kz[((long long)l * 2 + 1) * J + jj];
    const double2 bd = beta[(long long)l * 2 * J + jj], bu = beta[((long long)l * 2 + 1) * J + jj];
    for (int kk = 0; kk < nks; kk++) {
        if (kk < g.nk) {
            const double z = (double)zlist[g.zi[kk]];
            const float2 fd = phase_fp64(kd.x, kd.y, z - zb[l]);
            const float2 fu = phase_fp64(ku.x, ku.y, z - zb[l + 1]);
            const double dre = bd.x * fd.x - bd.y * fd.y, dim = bd.x * fd.y + bd.y * fd.x;
            const double ure = bu.x * fu.x - bu.y * fu.y, uim = bu.x * fu.y + bu.y * fu.x;
            out0[kk] = make_float2((float)(dre + ure), (float)(dim + uim));
            out1[kk] = make_float2((float)(dre - ure), (float)(dim - uim));
        } else {
            out0[kk] = make_float2(0.f, 0.f);
            out1[kk] = make_float2(0.f, 0.f);
        }
    }
}

// C[zi][c][p] = sum over the slice's modes of Q[l][h][c][p][j] * Phi[g][h'][j][kk]:
//   two-half sets (H = 2): h = h' = 0, 1 (downward and upward modes, 2J terms);
//   paired sets (H = 1): the one block V, h' = 0 for rows Ex, Ey and 1 for rows Ez (J terms).
//
// HBM-streaming contraction: one warp owns RW rows (c, p) at a time; its lanes read 2
// consecutive complex Q entries each (512 contiguous bytes per warp and row per step) and
// multiply them with the group's phases, staged in shared memory per chunk of kChunk modes
// and shared by the CTA's 8 warps.  Every CTA works on one component c (blockIdx.x / nbp),
// so its phase rows are the same for all its warps.  Lane partial sums are reduced with warp
// shuffles.
constexpr int kCtrWarps = 8;
constexpr int kCtrChunk = 1024;

// pipeline depth of the Q stream: stages x rows per warp = 16 float4 in flight per lane
template <int RW, int NK>
struct CtrCfg {
    static constexpr int kStages = NK == 8 ? 4 : (16 / RW < 2 ? 2 : 16 / RW);
    static constexpr size_t kSmem = (size_t)NK * (kCtrChunk / 2) * 16 + (size_t)kCtrWarps * kStages * RW * 32 * 16;
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <int NK, int RW>
__global__ void __launch_bounds__(kCtrWarps * 32, 2)
sep_contract_kernel(const PGroup* __restrict__ groups, const float2* __restrict__ Phi,
                    const float2* __restrict__ Q, int MF, int J, int H, float2* __restrict__ C) {
    constexpr int S = CtrCfg<RW, NK>::kStages;
    extern __shared__ float4 smem4[];
    // (phi[j][kk], phi[j+1][kk]) pairs per plane; then per lane S x RW private Q slots
    float4 (*ph)[kCtrChunk / 2] = reinterpret_cast<float4 (*)[kCtrChunk / 2]>(smem4);
    const PGroup g = groups[blockIdx.y];
    const int l = g.region - 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* qs = smem4 + NK * (kCtrChunk / 2) + (size_t)warp * S * RW * 32 + lane;   // slot (s, r): qs[(s*RW + r)*32]
    const int nbp = gridDim.x / 3;                       // CTAs per component
    const int c = blockIdx.x / nbp;
    const int p0 = ((blockIdx.x - c * nbp) * kCtrWarps + warp) * RW;
    float acc[RW][NK][2];
#pragma unroll
    for (int r = 0; r < RW; r++)
#pragma unroll
        for (int kk = 0; kk < NK; kk++) acc[r][kk][0] = acc[r][kk][1] = 0.f;
    const float2* Pg = Phi + (long long)blockIdx.y * 2 * J * NK;
    for (int half = 0; half < H; half++) {
        const int ph_half = H == 2 ? half : (c == 2 ? 1 : 0);
        const float4* qrow[RW];
#pragma unroll
        for (int r = 0; r < RW; r++) {
            const int p = min(p0 + r, MF - 1);            // rows past the end repeat the last (not written)
            qrow[r] = reinterpret_cast<const float4*>(Q + ((((long long)l * H + half) * 3 + c) * MF + p) * (long long)J);
        }
        for (int j0 = 0; j0 < J; j0 += kCtrChunk) {
            const int nj = min(kCtrChunk, J - j0);
            __syncthreads();
            // consecutive threads fill consecutive pairs of one plane (conflict-free stores)
            for (int e = threadIdx.x; e < (nj / 2) * NK; e += blockDim.x) {
                const int kk = e / (nj / 2), jp = e % (nj / 2);
                const float2 a = Pg[((long long)ph_half * J + j0 + 2 * jp) * NK + kk];
                const float2 b = Pg[((long long)ph_half * J + j0 + 2 * jp + 1) * NK + kk];
                ph[kk][jp] = make_float4(a.x, a.y, b.x, b.y);
            }
            __syncthreads();
            // lane iterations jp = lane + 32 it; the Q pairs of iteration it arrive through an
            // S-deep cp.async ring (the slot refilled at iteration it is the one read at it - 1)
            const int npair = nj / 2;
            const int nit = lane < npair ? (npair - lane + 31) / 32 : 0;
#pragma unroll
            for (int st = 0; st < S - 1; st++) {
                if (st < nit) {
                    const int jp = lane + 32 * st;
#pragma unroll
                    for (int r = 0; r < RW; r++) cp_async16(qs + (st * RW + r) * 32, qrow[r] + j0 / 2 + jp);
                }
                cp_async_commit();
            }
            for (int it = 0; it < nit; it++) {
                const int nxt = it + S - 1;
                if (nxt < nit) {
                    const int jp = lane + 32 * nxt, sl = nxt % S;
#pragma unroll
                    for (int r = 0; r < RW; r++) cp_async16(qs + (sl * RW + r) * 32, qrow[r] + j0 / 2 + jp);
                }
                cp_async_commit();
                cp_async_wait<S - 1>();
                const int jp = lane + 32 * it, sl = it % S;
                float4 f[NK];
#pragma unroll
                for (int kk = 0; kk < NK; kk++) f[kk] = ph[kk][jp];
#pragma unroll
                for (int r = 0; r < RW; r++) {
                    const float4 q = qs[(sl * RW + r) * 32];
#pragma unroll
                    for (int kk = 0; kk < NK; kk++) {
                        acc[r][kk][0] = fmaf(q.x, f[kk].x, fmaf(-q.y, f[kk].y, acc[r][kk][0]));
                        acc[r][kk][1] = fmaf(q.x, f[kk].y, fmaf(q.y, f[kk].x, acc[r][kk][1]));
                        acc[r][kk][0] = fmaf(q.z, f[kk].z, fmaf(-q.w, f[kk].w, acc[r][kk][0]));
                        acc[r][kk][1] = fmaf(q.z, f[kk].w, fmaf(q.w, f[kk].z, acc[r][kk][1]));
                    }
                }
            }
            cp_async_wait<0>();
        }
    }
#pragma unroll
    for (int r = 0; r < RW; r++) {
        const int p = p0 + r;
#pragma unroll
        for (int kk = 0; kk < NK; kk++) {
            float vr = acc[r][kk][0], vi = acc[r][kk][1];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                vr += __shfl_xor_sync(0xffffffffu, vr, o);
                vi += __shfl_xor_sync(0xffffffffu, vi, o);
            }
            if (lane == 0 && p < MF && kk < g.nk) C[((long long)g.zi[kk] * 3 + c) * MF + p] = make_float2(vr, vi);
        }
    }
}

// Exterior regions: region 0 = incident (referenced at the origin) + reflected (at z_0),
// last region = transmitted (at z_Z).  One thread per (z entry, c, p), FP64.
__global__ void sep_exterior_kernel(const int2* __restrict__ ext, int n_ext, const float* __restrict__ zlist,
                                    const double2* __restrict__ xd, int MF, double z0, double zZ,
                                    float2* __restrict__ C) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)n_ext * 3 * MF) return;
    const int e = (int)(idx / (3 * MF));
    const int rem = (int)(idx % (3 * MF));
    const int c = rem / MF, p = rem % MF;
    const int2 ent = ext[e];     // (zi, 0 = top exterior / 1 = bottom exterior)
    const double z = (double)zlist[ent.x];
    // xd layout: inc[3][MF], refl[3][MF], trans[3][MF], kz_inc[MF], kz_refl[MF], kz_trans[MF]
    const double2* inc = xd;
    const double2* refl = xd + 3 * MF;
    const double2* trans = xd + 6 * MF;
    const double2* kzi = xd + 9 * MF;
    const double2* kzr = xd + 10 * MF;
    const double2* kzt = xd + 11 * MF;
    double sr = 0.0, si = 0.0;
    auto add = [&](double2 a, double2 k, double dz) {
        const float2 f = phase_fp64(k.x, k.y, dz);
        sr += a.x * (double)f.x - a.y * (double)f.y;
        si += a.x * (double)f.y + a.y * (double)f.x;
    };
    if (ent.y == 0) {
        add(inc[c * MF + p], kzi[p], z);
        add(refl[c * MF + p], kzr[p], z - z0);
    } else {
        add(trans[c * MF + p], kzt[p], z - zZ);
    }
    C[((long long)ent.x * 3 + c) * MF + p] = make_float2((float)sr, (float)si);
}

// tab[m][i] = exp(i k_m x_i), x_i = s + d * i in float (one rounding per operation)
__global__ void sep_table_kernel(const double* __restrict__ k, int M, float s, float d, int N, float2* __restrict__ tab) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)M * N) return;
    const int m = (int)(idx / N), i = (int)(idx % N);
    const float x = __fadd_rn(s, __fmul_rn(d, (float)i));
    tab[idx] = phase_fp64(k[m], 0.0, (double)x);
}

// Stage 2a: T[r][c][m] = sum_n R(r, n) * C[zi(r)][c][p(m, n)]
//   ctype 0: m = a (keep), n = b (contract), p = a*M1 + b
//   ctype 1: m = b (keep), n = a (contract)
// R(r, n) = Rtab[n * rld + r % rmod];  zi(r) = zoff + r / rdiv
__global__ void sep_rows_kernel(const float2* __restrict__ C, const float2* __restrict__ Rtab, int rld, int rmod,
                                int rdiv, int zoff, int nrows, int ctype, int M0, int M1, float2* __restrict__ T) {
    const int Mk = ctype == 0 ? M0 : M1;
    const int Mn = ctype == 0 ? M1 : M0;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nrows * 3 * Mk) return;
    const int r = (int)(idx / (3 * Mk));
    const int rem = (int)(idx % (3 * Mk));
    const int c = rem / Mk, m = rem % Mk;
    const int zi = zoff + r / rdiv;
    const float2* Cz = C + ((long long)zi * 3 + c) * M0 * M1;
    const int ro = r % rmod;
    float sr = 0.f, si = 0.f;
    for (int n = 0; n < Mn; n++) {
        const float2 rv = Rtab[(long long)n * rld + ro];
        const float2 cv = ctype == 0 ? Cz[m * M1 + n] : Cz[n * M1 + m];
        sr = fmaf(rv.x, cv.x, fmaf(-rv.y, cv.y, sr));
        si = fmaf(rv.x, cv.y, fmaf(rv.y, cv.x, si));
    }
    T[idx] = make_float2(sr, si);
}

// Stage 2a for a volume: T[k*Ny + j][c][a] = sum_b Ey[b][j] C[k][c][a*M1 + b].
// One CTA per (z-plane k, block of kRowsBlk rows j): C[k] is staged transposed ([c][b][a],
// so lanes with consecutive a read consecutive words) with the block's Ey phases, also
// transposed ([b][row], 16-byte aligned).  Each thread computes a kRowsT x 2 block of outputs
// (rows j, two adjacent columns (c, a)): per harmonic b it loads the kRowsT row phases as
// kRowsT / 2 16-byte words (the same for the warp: broadcast) and two column values
// (consecutive across the warp) for 2 kRowsT complex multiply-adds.
constexpr int kRowsBlk = 64;
constexpr int kRowsT = 8;
// float2 offset of the row phases in the kernel's shared memory (16-byte aligned)
__host__ __device__ inline int rows_phase_off(int M0, int M1) { return (3 * M0 * M1 + 2 + 1) & ~1; }

__global__ void __launch_bounds__(256)
sep_rows_volume_kernel(const float2* __restrict__ C, const float2* __restrict__ tabY, int Ny, int M0, int M1,
                       float2* __restrict__ T) {
    extern __shared__ float2 sm2[];
    float2* sC = sm2;                              // [3][M1][M0] (+1 pad entry for odd M0)
    float2* sR = sm2 + rows_phase_off(M0, M1);     // [M1][kRowsBlk]
    const int k = blockIdx.y;
    const int j0 = blockIdx.x * kRowsBlk;
    const int MF = M0 * M1;
    const float2* Ck = C + (long long)k * 3 * MF;
    for (int e = threadIdx.x; e < 3 * MF; e += blockDim.x) {
        const int c = e / MF, p = e % MF, a = p / M1, b = p % M1;
        sC[(c * M1 + b) * M0 + a] = Ck[e];
    }
    if (threadIdx.x < 2) sC[3 * MF + threadIdx.x] = make_float2(0.f, 0.f);
    for (int e = threadIdx.x; e < kRowsBlk * M1; e += blockDim.x) {
        const int b = e / kRowsBlk, r = e % kRowsBlk;
        sR[e] = (j0 + r < Ny) ? tabY[(long long)b * Ny + j0 + r] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int ncol = 3 * M0;
    const int npair = (ncol + 1) / 2;
    const int nitems = (kRowsBlk / kRowsT) * npair;
    for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
        const int rb = it / npair, q = it % npair;
        const int r0 = rb * kRowsT;
        if (j0 + r0 >= Ny) continue;
        const int col0 = 2 * q, col1 = min(2 * q + 1, ncol - 1);
        const int c0 = col0 / M0, a0 = col0 % M0, c1 = col1 / M0, a1 = col1 % M0;
        const float2* cp0 = sC + c0 * M1 * M0 + a0;
        const float2* cp1 = sC + c1 * M1 * M0 + a1;
        const float4* rp = reinterpret_cast<const float4*>(sR + r0);
        float acc[kRowsT][2][2];
#pragma unroll
        for (int i = 0; i < kRowsT; i++) acc[i][0][0] = acc[i][0][1] = acc[i][1][0] = acc[i][1][1] = 0.f;
        for (int b = 0; b < M1; b++) {
            const float2 v0 = cp0[b * M0], v1 = cp1[b * M0];
            float2 rvs[kRowsT];
#pragma unroll
            for (int i2 = 0; i2 < kRowsT / 2; i2++) {
                const float4 w = rp[b * (kRowsBlk / 2) + i2];
                rvs[2 * i2] = make_float2(w.x, w.y);
                rvs[2 * i2 + 1] = make_float2(w.z, w.w);
            }
#pragma unroll
            for (int i = 0; i < kRowsT; i++) {
                const float2 rv = rvs[i];
                acc[i][0][0] = fmaf(rv.x, v0.x, fmaf(-rv.y, v0.y, acc[i][0][0]));
                acc[i][0][1] = fmaf(rv.x, v0.y, fmaf(rv.y, v0.x, acc[i][0][1]));
                acc[i][1][0] = fmaf(rv.x, v1.x, fmaf(-rv.y, v1.y, acc[i][1][0]));
                acc[i][1][1] = fmaf(rv.x, v1.y, fmaf(rv.y, v1.x, acc[i][1][1]));
            }
        }
#pragma unroll
        for (int i = 0; i < kRowsT; i++) {
            const int j = j0 + r0 + i;
            if (j >= Ny) break;
            float2* trow = T + ((long long)k * Ny + j) * 3 * M0;
            trow[c0 * M0 + a0] = make_float2(acc[i][0][0], acc[i][0][1]);
            if (col1 != col0) trow[c1 * M0 + a1] = make_float2(acc[i][1][0], acc[i][1][1]);
        }
    }
}

// Stage 2b (FP32 SIMT): E[r][col][c] = sum_m T[r][c][m] * F[m][col]
// CTA: 32 rows x 64 columns; thread: 2 rows x 4 columns x 3 components.
constexpr int kSynRows = 32, kSynCols = 64, kSynMaxK = 64;

__global__ void __launch_bounds__(256)
sep_synth_kernel(const float2* __restrict__ T, const float2* __restrict__ F, int nrows, int ncols, int Mk,
                 float* __restrict__ out) {
    extern __shared__ float2 smem[];
    float2* sT = smem;                                  // [kSynRows][3][Mk]
    float2* sF = smem + kSynRows * 3 * kSynMaxK;        // [Mk][kSynCols]
    const int r0 = blockIdx.y * kSynRows, c0 = blockIdx.x * kSynCols;
    for (int e = threadIdx.x; e < kSynRows * 3 * Mk; e += blockDim.x) {
        const int rr = e / (3 * Mk);
        sT[e] = (r0 + rr < nrows) ? T[(long long)r0 * 3 * Mk + e] : make_float2(0.f, 0.f);
    }
    for (int e = threadIdx.x; e < Mk * kSynCols; e += blockDim.x) {
        const int m = e / kSynCols, cc = e % kSynCols;
        sF[e] = (c0 + cc < ncols) ? F[(long long)m * ncols + c0 + cc] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int tr = threadIdx.x / 16, tc = threadIdx.x % 16;
    float acc[2][4][3][2];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 4; b++)
#pragma unroll
            for (int c = 0; c < 3; c++) acc[a][b][c][0] = acc[a][b][c][1] = 0.f;
    for (int m = 0; m < Mk; m++) {
        float2 f[4];
#pragma unroll
        for (int b = 0; b < 4; b++) f[b] = sF[m * kSynCols + tc + 16 * b];
#pragma unroll
        for (int a = 0; a < 2; a++) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const float2 t = sT[((tr * 2 + a) * 3 + c) * Mk + m];
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    acc[a][b][c][0] = fmaf(t.x, f[b].x, fmaf(-t.y, f[b].y, acc[a][b][c][0]));
                    acc[a][b][c][1] = fmaf(t.x, f[b].y, fmaf(t.y, f[b].x, acc[a][b][c][1]));
                }
            }
        }
    }
#pragma unroll
    for (int a = 0; a < 2; a++) {
        const int r = r0 + tr * 2 + a;
        if (r >= nrows) continue;
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int col = c0 + tc + 16 * b;
            if (col >= ncols) continue;
            float* o = out + ((long long)r * ncols + col) * 6;
            const float2 v0 = make_float2(acc[a][b][0][0], acc[a][b][0][1]);
            const float2 v1 = make_float2(acc[a][b][1][0], acc[a][b][1][1]);
            const float2 v2 = make_float2(acc[a][b][2][0], acc[a][b][2][1]);
            reinterpret_cast<float2*>(o)[0] = v0;
            reinterpret_cast<float2*>(o)[1] = v1;
            reinterpret_cast<float2*>(o)[2] = v2;
        }
    }
}

// ------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------
static int64_t sep_region(const scw_sep_s* s, float z) {
    int64_t l = 0;
    const double zd = (double)z;
    for (int li = 0; li <= s->Z; li++) {
        const double thr = (s->rule == 0) ? (double)s->z_layers[li] - 0.001 : (double)s->z_layers[li];
        if (zd >= thr) l = li + 1;
    }
    return l;
}

static float host_coord(float s, float d, int i) {
    volatile float p = d * (float)i;
    volatile float r = s + p;
    return r;
}

static size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// Stage-1 plan: the z-planes grouped by region (up to kMaxGroup planes of one region share a
// pass over that region's Q), exterior planes listed apart.
static void stage1_plan(const scw_sep_s* s, SepEvalPlan& p) {
    std::map<int64_t, std::vector<int>> by_region;
    for (int i = 0; i < (int)p.zlist.size(); i++) by_region[sep_region(s, p.zlist[i])].push_back(i);
    p.max_nk = 1;
    p.groups.clear();
    p.ext.clear();
    for (auto& kv : by_region) {
        const int64_t r = kv.first;
        if (r == 0 || r == s->Z + 1) {
            for (int zi : kv.second) p.ext.push_back(make_int2(zi, r == 0 ? 0 : 1));
            continue;
        }
        for (size_t o = 0; o < kv.second.size(); o += kMaxGroup) {
            PGroup g{};
            g.region = (int)r;
            g.nk = (int)std::min<size_t>(kMaxGroup, kv.second.size() - o);
            for (int kk = 0; kk < g.nk; kk++) g.zi[kk] = kv.second[o + kk];
            p.max_nk = std::max(p.max_nk, g.nk);
            p.groups.push_back(g);
        }
    }
    const size_t gbytes = p.groups.size() * sizeof(PGroup), ebytes = p.ext.size() * sizeof(int2),
                 zbytes = p.zlist.size() * sizeof(float);
    p.off_e = align256(gbytes);
    p.off_z = p.off_e + align256(ebytes);
    p.desc_bytes = p.off_z + align256(zbytes);
}

void sep_eval_desc(const SepEvalPlan& p, char* h) {
    if (!p.groups.empty()) std::memcpy(h, p.groups.data(), p.groups.size() * sizeof(PGroup));
    if (!p.ext.empty()) std::memcpy(h + p.off_e, p.ext.data(), p.ext.size() * sizeof(int2));
    std::memcpy(h + p.off_z, p.zlist.data(), p.zlist.size() * sizeof(float));
}

// Stage 1 for the plan's z-values: fills C [nz][3][MF]; descriptors already on the device.
static scw_status stage1_record(scw_sep s, const SepEvalPlan& p, const char* d_desc, float2* dC, char* cursor) {
    scw_ctx ctx = s->ctx;
    const int MF = s->MF, J = s->Jp;          // device row stride (even)
    const auto& groups = p.groups;
    const auto& ext = p.ext;
    const int max_nk = p.max_nk;
    const PGroup* dg = (const PGroup*)d_desc;
    const int2* de = (const int2*)(d_desc + p.off_e);
    const float* dz = (const float*)(d_desc + p.off_z);
    if (!groups.empty()) {
        if (J > 0) {
            const int nks = max_nk <= 1 ? 1 : max_nk <= 2 ? 2 : max_nk <= 4 ? 4 : 8;
            float2* dPhi = (float2*)cursor;
            cursor += align256(groups.size() * 2 * (size_t)J * nks * sizeof(float2));
            // one thread per (half, mode) for a two-half set, per mode for a paired set
            dim3 gp(((s->halves == 1 ? J : 2 * J) + 255) / 256, (unsigned)groups.size());
            {
                LaunchTimer lt(ctx, "sep_phase_kernel");
                sep_phase_kernel<<<gp, 256, 0, ctx->stream>>>(dg, dz, s->dKz, s->halves == 1 ? s->dBeta : nullptr,
                                                              s->dzb, J, nks, dPhi);
            }
            SCW_CUDA_TRY(cudaGetLastError());
            ctx->launches++;
            // per component c, ceil(MF / (warps x rows per warp)) CTAs
            auto grid_for = [&](int rw) {
                return dim3(3 * ((MF + kCtrWarps * rw - 1) / (kCtrWarps * rw)), (unsigned)groups.size());
            };
            LaunchTimer lt(ctx, "sep_contract_kernel");
            auto launch = [&](auto kernel, int rw, size_t smem) -> scw_status {
                SCW_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                kernel<<<grid_for(rw), kCtrWarps * 32, smem, ctx->stream>>>(dg, dPhi, s->dQ, MF, J, s->halves, dC);
                return SCW_OK;
            };
            scw_status ls;
            if (s->ctr_shape == 0) {
                if (nks == 1) ls = launch(sep_contract_kernel<1, 8>, 8, CtrCfg<8, 1>::kSmem);
                else if (nks == 2) ls = launch(sep_contract_kernel<2, 8>, 8, CtrCfg<8, 2>::kSmem);
                else if (nks == 4) ls = launch(sep_contract_kernel<4, 4>, 4, CtrCfg<4, 4>::kSmem);
                else ls = launch(sep_contract_kernel<8, 2>, 2, CtrCfg<2, 8>::kSmem);
            } else {
                if (nks == 1) ls = launch(sep_contract_kernel<1, 4>, 4, CtrCfg<4, 1>::kSmem);
                else if (nks == 2) ls = launch(sep_contract_kernel<2, 4>, 4, CtrCfg<4, 2>::kSmem);
                else if (nks == 4) ls = launch(sep_contract_kernel<4, 2>, 2, CtrCfg<2, 4>::kSmem);
                else ls = launch(sep_contract_kernel<8, 1>, 1, CtrCfg<1, 8>::kSmem);
            }
            if (ls != SCW_OK) return ls;
            SCW_CUDA_TRY(cudaGetLastError());
            ctx->launches++;
        } else {
            // no interior waves (--external files): interior coefficients are zero
            for (const auto& g : groups)
                for (int kk = 0; kk < g.nk; kk++)
                    SCW_CUDA_TRY(cudaMemsetAsync(dC + (size_t)g.zi[kk] * 3 * MF, 0, 3 * MF * sizeof(float2),
                                                 ctx->stream));
        }
    }
    if (!ext.empty()) {
        const long long n = (long long)ext.size() * 3 * MF;
        LaunchTimer lt(ctx, "sep_exterior_kernel");
        sep_exterior_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(de, (int)ext.size(), dz, s->dExt, MF,
                                                                                 s->zb[0], s->zb[s->Z], dC);
        SCW_CUDA_TRY(cudaGetLastError());
        ctx->launches++;
    }
    return SCW_OK;
}

static scw_status launch_table(scw_ctx ctx, const double* dk, int M, float st, float d, int N, float2* tab) {
    const long long n = (long long)M * N;
    LaunchTimer lt(ctx, "sep_table_kernel");
    sep_table_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(dk, M, st, d, N, tab);
    SCW_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    return SCW_OK;
}

static scw_status launch_rows(scw_ctx ctx, const float2* C, const float2* Rtab, int rld, int rmod, int rdiv, int zoff,
                              int nrows, int ctype, int M0, int M1, float2* T) {
    const int Mk = ctype == 0 ? M0 : M1;
    const long long n = (long long)nrows * 3 * Mk;
    LaunchTimer lt(ctx, "sep_rows_kernel");
    sep_rows_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(C, Rtab, rld, rmod, rdiv, zoff, nrows, ctype,
                                                                          M0, M1, T);
    SCW_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    return SCW_OK;
}

scw_status sep_synth(scw_ctx ctx, const float2* T, const float2* F, int nrows, int ncols, int Mk, float* out,
                     int method) {
    if (method == SCW_SEP_TF32X3 || method == SCW_SEP_BF16X3) {
        // shapes whose operands do not fit the tensor-core kernel's shared and tensor memory (more
        // than 48 harmonics along the synthesis axis for 3xTF32, 80 for split-BF16) run the FP32
        // SIMT GEMM below, which is at least as accurate
        scw_status st = sep_synth_tc(ctx, T, F, nrows, ncols, Mk, out, method);
        if (st != SCW_ERR_UNSUPPORTED) return st;
    }
    if (Mk > kSynMaxK) return fail(SCW_ERR_UNSUPPORTED, "more than 64 harmonics along the synthesis axis");
    const size_t smem = (size_t)(kSynRows * 3 * kSynMaxK + kSynMaxK * kSynCols) * sizeof(float2);
    static bool attr_set = false;
    if (!attr_set) {
        SCW_CUDA_TRY(cudaFuncSetAttribute(sep_synth_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = true;
    }
    dim3 grid((ncols + kSynCols - 1) / kSynCols, (nrows + kSynRows - 1) / kSynRows);
    LaunchTimer lt(ctx, "sep_synth_kernel");
    sep_synth_kernel<<<grid, 256, smem, ctx->stream>>>(T, F, nrows, ncols, Mk, out);
    SCW_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    return SCW_OK;
}

// Sizes and stage-1 grouping of a plan whose kind, geometry and z-list are set.
static scw_status sep_plan_finish(const scw_sep_s* s, SepEvalPlan& p) {
    const int M0 = s->M0, M1 = s->M1, MF = s->MF;
    const int nz = (int)p.zlist.size();
    if (p.kind == 0) { p.nrows = p.Nz * p.Nb; p.ncols = p.Na; p.Mk = M0; }
    else if (p.kind == 1) { p.nrows = p.Nb; p.ncols = p.Na; p.Mk = M0; }
    else { p.nrows = p.Nb; p.ncols = p.Na; p.Mk = M1; }
    if (p.kind == 0) {
        const size_t smem = (size_t)(3 * M0 * M1 + 2 + kRowsBlk * M1) * sizeof(float2);
        if (smem > 200 * 1024) return fail(SCW_ERR_UNSUPPORTED, "harmonic grid too large for the row stage");
    }
    // phases for the PGroups: at most nz groups
    p.phi_bytes = align256((size_t)nz * 2 * (size_t)s->Jp * kMaxGroup * sizeof(float2));
    p.c_bytes = align256((size_t)nz * 3 * MF * sizeof(float2));
    // slack past the last row: the tensor-core producer reads whole 16-row tiles of T
    p.t_bytes = align256((size_t)p.nrows * 3 * p.Mk * sizeof(float2) + 16 * 3 * 64 * sizeof(float2) + 4096);
    p.tab_bytes = align256((size_t)(M0 + M1) * (p.Na + p.Nb + 2) * sizeof(float2));
    p.scratch_bytes = p.phi_bytes + p.c_bytes + p.t_bytes + 2 * p.tab_bytes;
    stage1_plan(s, p);
    return SCW_OK;
}

static void sep_plan_geom(SepEvalPlan& p, int kind, float a0, float b0, float c, float da, float db, float dz, int Na,
                          int Nb, int Nz, int method) {
    p.kind = kind;
    p.a0 = a0;
    p.b0 = b0;
    p.c = c;
    p.da = da;
    p.db = db;
    p.dz = dz;
    p.Na = Na;
    p.Nb = Nb;
    p.Nz = Nz;
    p.method = method;
    p.zlist.clear();
}

// One evaluation "sheet" family: a volume of xy planes, or an xz / yz plane.  Host-only plan.
scw_status sep_eval_plan(const scw_sep_s* s, int kind, float a0, float b0, float c, float da, float db, float dz,
                         int Na, int Nb, int Nz, int method, SepEvalPlan& p) {
    sep_plan_geom(p, kind, a0, b0, c, da, db, dz, Na, Nb, Nz, method);
    if (kind == 0) {            // volume: Nz xy planes at z = c + dz*k; a = x (Na), b = y (Nb)
        for (int k = 0; k < Nz; k++) p.zlist.push_back(host_coord(c, dz, k));
    } else {                    // kind 1: xz plane at y = c (a = x, rows = z); kind 2: yz plane at x = c (a = y)
        for (int k = 0; k < Nb; k++) p.zlist.push_back(host_coord(b0, db, k));
    }
    return sep_plan_finish(s, p);
}

// Plan of the xy planes k0 .. k1-1 of the volume (x_start, y_start, z_start, dx, dy, dz): the
// planes keep the z-values the whole volume's plan gives them.
static scw_status sep_eval_plan_planes(const scw_sep_s* s, float a0, float b0, float z_start, float da, float db,
                                       float dz, int Na, int Nb, int k0, int k1, int method, SepEvalPlan& p) {
    sep_plan_geom(p, 0, a0, b0, z_start, da, db, dz, Na, Nb, k1 - k0, method);
    for (int k = k0; k < k1; k++) p.zlist.push_back(host_coord(z_start, dz, k));
    return sep_plan_finish(s, p);
}

// Planes k_begin .. k_end-1 of a volume into device memory, with the z-values the whole volume has.
scw_status sep_eval_slab(scw_sep s, float x0, float y0, float z0, float dx, float dy, float dz, int Nx, int Ny,
                         int k_begin, int k_end, float* dE, int method);

// Stage 2 of one planned evaluation (tables, row products, output GEMM) on the context stream;
// scratch laid out as in sep_eval_record (C, T, two tables, then stage 1's work).
static scw_status stage2_record(scw_sep s, const SepEvalPlan& p, char* scratch, float* dE) {
    scw_ctx ctx = s->ctx;
    const int M0 = s->M0, M1 = s->M1;
    char* cursor = scratch;
    float2* dC = (float2*)cursor;
    cursor += p.c_bytes;
    float2* dT = (float2*)cursor;
    cursor += p.t_bytes;
    float2* tabA = (float2*)cursor;
    cursor += p.tab_bytes;
    float2* tabB = (float2*)cursor;
    cursor += p.tab_bytes;
    scw_status st = SCW_OK;
    const int nrows = p.nrows, ncols = p.ncols, Mk = p.Mk, Na = p.Na, Nb = p.Nb, Nz = p.Nz;
    if (p.kind == 0) {
        // F = Ex table [a][x]; R = Ey table [b][y]
        if ((st = launch_table(ctx, s->dkx, M0, p.a0, p.da, Na, tabA)) != SCW_OK) return st;
        if ((st = launch_table(ctx, s->dky, M1, p.b0, p.db, Nb, tabB)) != SCW_OK) return st;
        {
            const size_t smem = (size_t)(rows_phase_off(M0, M1) + kRowsBlk * M1) * sizeof(float2);
            SCW_CUDA_TRY(cudaFuncSetAttribute(sep_rows_volume_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem));
            dim3 grid((Nb + kRowsBlk - 1) / kRowsBlk, Nz);
            LaunchTimer lt(ctx, "sep_rows_volume_kernel");
            sep_rows_volume_kernel<<<grid, 256, smem, ctx->stream>>>(dC, tabB, Nb, M0, M1, dT);
            SCW_CUDA_TRY(cudaGetLastError());
            ctx->launches++;
        }
        return sep_synth(ctx, dT, tabA, nrows, ncols, Mk, dE, p.method);
    } else if (p.kind == 1) {
        // xz plane at y = c: R = Ey(c) [b]; F = Ex table [a][x]
        if ((st = launch_table(ctx, s->dkx, M0, p.a0, p.da, Na, tabA)) != SCW_OK) return st;
        if ((st = launch_table(ctx, s->dky, M1, p.c, 0.f, 1, tabB)) != SCW_OK) return st;
        if ((st = launch_rows(ctx, dC, tabB, 1, 1, 1, 0, nrows, 0, M0, M1, dT)) != SCW_OK) return st;
        return sep_synth(ctx, dT, tabA, nrows, ncols, Mk, dE, p.method);
    } else {
        // yz plane at x = c: R = Ex(c) [a]; F = Ey table [b][y]
        if ((st = launch_table(ctx, s->dky, M1, p.a0, p.da, Na, tabA)) != SCW_OK) return st;
        if ((st = launch_table(ctx, s->dkx, M0, p.c, 0.f, 1, tabB)) != SCW_OK) return st;
        if ((st = launch_rows(ctx, dC, tabB, 1, 1, 1, 0, nrows, 1, M0, M1, dT)) != SCW_OK) return st;
        return sep_synth(ctx, dT, tabA, nrows, ncols, Mk, dE, p.method);
    }
}

// Launches of one planned evaluation (no allocation, no host synchronisation).
scw_status sep_eval_record(scw_sep s, const SepEvalPlan& p, const char* d_desc, char* scratch, float* dE) {
    const size_t head = p.c_bytes + p.t_bytes + 2 * p.tab_bytes;
    scw_status st = stage1_record(s, p, d_desc, (float2*)scratch, scratch + head);
    if (st != SCW_OK) return st;
    return stage2_record(s, p, scratch, dE);
}

scw_status sep_eval(scw_sep s, int kind, float a0, float b0, float c, float da, float db, float dz, int Na, int Nb,
                    int Nz, float* dE, int method) {
    scw_ctx ctx = s->ctx;
    SCW_ON_DEVICE(ctx->device);
    SepEvalPlan p;
    scw_status st = sep_eval_plan(s, kind, a0, b0, c, da, db, dz, Na, Nb, Nz, method, p);
    if (st != SCW_OK) return st;
    if ((st = ctx->sep_scratch.reserve(p.scratch_bytes)) != SCW_OK) return st;
    // descriptors to the device (pinned staging, guarded by the context's event)
    SCW_CUDA_TRY(cudaEventSynchronize(ctx->desc_done));
    if ((st = ctx->host_desc.reserve(p.desc_bytes)) != SCW_OK) return st;
    if ((st = ctx->desc.reserve(p.desc_bytes)) != SCW_OK) return st;
    sep_eval_desc(p, (char*)ctx->host_desc.ptr);
    SCW_CUDA_TRY(cudaMemcpyAsync(ctx->desc.ptr, ctx->host_desc.ptr, p.desc_bytes, cudaMemcpyHostToDevice, ctx->stream));
    SCW_CUDA_TRY(cudaEventRecord(ctx->desc_done, ctx->stream));
    return sep_eval_record(s, p, (const char*)ctx->desc.ptr, (char*)ctx->sep_scratch.ptr, dE);
}


// ------------------------------------------------------------------------------------
// Host-streamed volume evaluation: the interior amplitudes come from host memory on every
// call.  Three streams overlap the link and the kernels: slices go up on the set's upload
// stream, each run of planes is evaluated on the context stream as soon as its slices are
// in, and each finished slab of planes goes down on the set's download stream.
// ------------------------------------------------------------------------------------
constexpr int kSlabSlots = 3;                         // output slabs in flight
constexpr size_t kSlabTarget = 64ull << 20;           // default bytes of output per run (at least one plane)
constexpr size_t kChunkTarget = 192ull << 20;         // default bytes of Q per upload chunk (at least one slice)

static scw_status stream_res(scw_sep s, size_t n_events, size_t slab_bytes) {
    if (!s->up_stream) SCW_CUDA_TRY(cudaStreamCreateWithFlags(&s->up_stream, cudaStreamNonBlocking));
    if (!s->down_stream) SCW_CUDA_TRY(cudaStreamCreateWithFlags(&s->down_stream, cudaStreamNonBlocking));
    while (s->events.size() < n_events) {
        cudaEvent_t e;
        SCW_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        s->events.push_back(e);
    }
    if (s->slab_bytes < slab_bytes) {
        if (s->dslab) cudaFree(s->dslab);
        s->dslab = nullptr;
        s->slab_bytes = 0;
        if (cudaMalloc(&s->dslab, slab_bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(SCW_ERR_NOMEM, "cudaMalloc of the output slabs");
        }
        s->slab_bytes = slab_bytes;
    }
    return SCW_OK;
}

struct StreamRun {
    int k0, k1;      // planes of the volume
    int chunk;       // upload chunk the run waits for (-1: exterior planes, no amplitudes needed)
};

// planes k_begin .. k_end-1 of the volume into Eh (plane k at Eh + (k - k_begin) planes)
scw_status sep_eval_volume_host(scw_sep s, const float2* Qh, float x0, float y0, float z0, float dx, float dy,
                                float dz, int Nx, int Ny, int k_begin, int k_end, float* Eh, int method) {
    scw_ctx ctx = s->ctx;
    SCW_ON_DEVICE(ctx->device);
    const size_t plane_bytes = (size_t)Nx * Ny * 6 * sizeof(float);
    const size_t J = (size_t)s->J, Jp = (size_t)s->Jp, MF = (size_t)s->MF;
    const size_t H = (size_t)s->halves;
    const size_t slice_bytes = H * 3 * MF * J * sizeof(float2);          // host layout [H][3][MF][J]
    const size_t chunk_target = s->chunk_bytes > 0 ? s->chunk_bytes : kChunkTarget;
    const size_t slab_target = s->slab_target > 0 ? s->slab_target : kSlabTarget;
    const int per_chunk = (int)std::max<size_t>(1, chunk_target / std::max<size_t>(slice_bytes, 1));
    const int max_run = (int)std::max<size_t>(1, slab_target / plane_bytes);
    // runs: consecutive planes in the same upload chunk, at most max_run planes each
    std::vector<StreamRun> runs;
    for (int k = k_begin; k < k_end; k++) {
        const int64_t r = sep_region(s, host_coord(z0, dz, k));
        const int ch = (r == 0 || r == s->Z + 1 || J == 0) ? -1 : (int)((r - 1) / per_chunk);
        if (!runs.empty() && runs.back().chunk == ch && runs.back().k1 == k && k - runs.back().k0 < max_run)
            runs.back().k1 = k + 1;
        else
            runs.push_back(StreamRun{k, k + 1, ch});
    }
    // chunks in the order the runs first need them
    const int n_chunks = s->Z > 0 ? (s->Z + per_chunk - 1) / per_chunk : 0;
    std::vector<int> order, ev_up(n_chunks, -1);
    for (const auto& rn : runs)
        if (rn.chunk >= 0 && ev_up[rn.chunk] < 0) {
            ev_up[rn.chunk] = (int)order.size();
            order.push_back(rn.chunk);
        }
    // plans and their descriptors (all uploaded at once, before the first launch)
    std::vector<SepEvalPlan> plans(runs.size());
    std::vector<size_t> desc_off(runs.size());
    size_t desc_total = 0, scratch = 0;
    int max_planes = 1;
    for (size_t i = 0; i < runs.size(); i++) {
        scw_status st = sep_eval_plan_planes(s, x0, y0, z0, dx, dy, dz, Nx, Ny, runs[i].k0, runs[i].k1, method,
                                             plans[i]);
        if (st != SCW_OK) return st;
        desc_off[i] = desc_total;
        desc_total += align256(plans[i].desc_bytes);
        scratch = std::max(scratch, plans[i].scratch_bytes);
        max_planes = std::max(max_planes, runs[i].k1 - runs[i].k0);
    }
    const size_t slab = align256((size_t)max_planes * plane_bytes);
    // events: [0] start, then one per chunk upload, then computed / downloaded per run
    const size_t n_ev = 1 + order.size() + 2 * runs.size();
    scw_status st = stream_res(s, n_ev, kSlabSlots * slab);
    if (st != SCW_OK) return st;
    if ((st = ctx->sep_scratch.reserve(scratch)) != SCW_OK) return st;
    SCW_CUDA_TRY(cudaEventSynchronize(ctx->desc_done));
    if ((st = ctx->host_desc.reserve(desc_total)) != SCW_OK) return st;
    if ((st = ctx->desc.reserve(desc_total)) != SCW_OK) return st;
    for (size_t i = 0; i < runs.size(); i++) sep_eval_desc(plans[i], (char*)ctx->host_desc.ptr + desc_off[i]);
    SCW_CUDA_TRY(cudaMemcpyAsync(ctx->desc.ptr, ctx->host_desc.ptr, desc_total, cudaMemcpyHostToDevice, ctx->stream));
    SCW_CUDA_TRY(cudaEventRecord(ctx->desc_done, ctx->stream));
    cudaEvent_t* ev = s->events.data();
    cudaEvent_t* ev_chunk = ev + 1;
    cudaEvent_t* ev_comp = ev + 1 + order.size();
    cudaEvent_t* ev_down = ev_comp + runs.size();
    // the amplitudes on the device are overwritten only after the work queued before this call
    SCW_CUDA_TRY(cudaEventRecord(ev[0], ctx->stream));
    SCW_CUDA_TRY(cudaStreamWaitEvent(s->up_stream, ev[0], 0));
    SCW_CUDA_TRY(cudaStreamWaitEvent(s->down_stream, ev[0], 0));
    for (size_t c = 0; c < order.size(); c++) {
        const int l0 = order[c] * per_chunk, l1 = std::min(s->Z, l0 + per_chunk);
        for (int l = l0; l < l1; l++) {
            const float2* src = Qh + (size_t)l * H * 3 * MF * J;
            float2* dst = s->dQ + (size_t)l * H * 3 * MF * Jp;
            if (J == Jp)
                SCW_CUDA_TRY(cudaMemcpyAsync(dst, src, slice_bytes, cudaMemcpyHostToDevice, s->up_stream));
            else
                SCW_CUDA_TRY(cudaMemcpy2DAsync(dst, Jp * sizeof(float2), src, J * sizeof(float2), J * sizeof(float2),
                                               H * 3 * MF, cudaMemcpyHostToDevice, s->up_stream));
        }
        SCW_CUDA_TRY(cudaEventRecord(ev_chunk[c], s->up_stream));
    }
    const char* d_desc = (const char*)ctx->desc.ptr;
    for (size_t i = 0; i < runs.size(); i++) {
        if (runs[i].chunk >= 0) SCW_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ev_chunk[ev_up[runs[i].chunk]], 0));
        if (i >= (size_t)kSlabSlots) SCW_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ev_down[i - kSlabSlots], 0));
        float* slot = (float*)((char*)s->dslab + (i % kSlabSlots) * slab);
        if ((st = sep_eval_record(s, plans[i], d_desc + desc_off[i], (char*)ctx->sep_scratch.ptr, slot)) != SCW_OK)
            return st;
        SCW_CUDA_TRY(cudaEventRecord(ev_comp[i], ctx->stream));
        SCW_CUDA_TRY(cudaStreamWaitEvent(s->down_stream, ev_comp[i], 0));
        SCW_CUDA_TRY(cudaMemcpyAsync((char*)Eh + (size_t)(runs[i].k0 - k_begin) * plane_bytes, slot,
                                     (size_t)(runs[i].k1 - runs[i].k0) * plane_bytes, cudaMemcpyDeviceToHost,
                                     s->down_stream));
        SCW_CUDA_TRY(cudaEventRecord(ev_down[i], s->down_stream));
    }
    SCW_CUDA_TRY(cudaStreamSynchronize(s->down_stream));
    SCW_CUDA_TRY(cudaStreamSynchronize(s->up_stream));
    return scw_ctx_synchronize(ctx);
}

// Planes k_begin .. k_end-1 in s->pipe_chunks chunks: stage 1 (phases, contraction; HBM reads)
// of chunk c on the context stream while stage 2 (row products, output GEMM; tensor cores and HBM
// writes) of chunk c - 1 runs on a high-priority stream, its output GEMM on sm_count /
// pipe_synth_div SMs so that the contraction keeps the rest.  Two scratch sets alternate between
// the chunks.  Every plane is computed exactly as by the one-pass form (its sums do not depend
// on the grouping or the grid).  Off by default (scw_sep_set_pipeline).
constexpr int kPipeMinPlanes = 32;

static scw_status sep_eval_slab_pipelined(scw_sep s, float x0, float y0, float z0, float dx, float dy, float dz,
                                          int Nx, int Ny, int k_begin, int k_end, float* dE, int method) {
    scw_ctx ctx = s->ctx;
    const int n = k_end - k_begin;
    const int per = (n + s->pipe_chunks - 1) / s->pipe_chunks;
    std::vector<SepEvalPlan> plans;
    std::vector<int> kb;
    for (int a = k_begin; a < k_end; a += per) {
        plans.emplace_back();
        kb.push_back(a);
        scw_status st = sep_eval_plan_planes(s, x0, y0, z0, dx, dy, dz, Nx, Ny, a, std::min(k_end, a + per), method,
                                             plans.back());
        if (st != SCW_OK) return st;
    }
    const int nc = (int)plans.size();
    std::vector<size_t> desc_off(nc);
    size_t desc_total = 0, scratch = 0;
    for (int c = 0; c < nc; c++) {
        desc_off[c] = desc_total;
        desc_total += align256(plans[c].desc_bytes);
        scratch = std::max(scratch, align256(plans[c].scratch_bytes));
    }
    if (!s->hi_stream) {
        int least = 0, greatest = 0;
        SCW_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        SCW_CUDA_TRY(cudaStreamCreateWithPriority(&s->hi_stream, cudaStreamNonBlocking, greatest));
    }
    while (s->pevents.size() < (size_t)(2 * nc + 1)) {
        cudaEvent_t e;
        SCW_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        s->pevents.push_back(e);
    }
    scw_status st = ctx->sep_scratch.reserve(2 * scratch);
    if (st != SCW_OK) return st;
    SCW_CUDA_TRY(cudaEventSynchronize(ctx->desc_done));
    if ((st = ctx->host_desc.reserve(desc_total)) != SCW_OK) return st;
    if ((st = ctx->desc.reserve(desc_total)) != SCW_OK) return st;
    for (int c = 0; c < nc; c++) sep_eval_desc(plans[c], (char*)ctx->host_desc.ptr + desc_off[c]);
    SCW_CUDA_TRY(cudaMemcpyAsync(ctx->desc.ptr, ctx->host_desc.ptr, desc_total, cudaMemcpyHostToDevice, ctx->stream));
    SCW_CUDA_TRY(cudaEventRecord(ctx->desc_done, ctx->stream));
    cudaEvent_t* ev1 = s->pevents.data() + 1;           // stage 1 of chunk c done
    cudaEvent_t* ev2 = ev1 + nc;                         // stage 2 of chunk c done
    SCW_CUDA_TRY(cudaEventRecord(s->pevents[0], ctx->stream));
    SCW_CUDA_TRY(cudaStreamWaitEvent(s->hi_stream, s->pevents[0], 0));
    const size_t plane_floats = (size_t)Nx * Ny * 6;
    const cudaStream_t main_stream = ctx->stream;
    for (int c = 0; c < nc; c++) {
        const SepEvalPlan& p = plans[c];
        char* buf = (char*)ctx->sep_scratch.ptr + (size_t)(c & 1) * scratch;
        if (c >= 2) SCW_CUDA_TRY(cudaStreamWaitEvent(main_stream, ev2[c - 2], 0));
        const size_t head = p.c_bytes + p.t_bytes + 2 * p.tab_bytes;
        if ((st = stage1_record(s, p, (const char*)ctx->desc.ptr + desc_off[c], (float2*)buf, buf + head)) != SCW_OK)
            return st;
        SCW_CUDA_TRY(cudaEventRecord(ev1[c], main_stream));
        SCW_CUDA_TRY(cudaStreamWaitEvent(s->hi_stream, ev1[c], 0));
        // stage 2 on the high-priority stream, its output GEMM on half the SMs
        ctx->stream = s->hi_stream;
        ctx->synth_ctas = std::max(1, ctx->sm_count / std::max(1, s->pipe_synth_div));
        st = stage2_record(s, p, buf, dE + (size_t)(kb[c] - k_begin) * plane_floats);
        ctx->stream = main_stream;
        ctx->synth_ctas = 0;
        if (st != SCW_OK) return st;
        SCW_CUDA_TRY(cudaEventRecord(ev2[c], s->hi_stream));
    }
    SCW_CUDA_TRY(cudaStreamWaitEvent(main_stream, ev2[nc - 1], 0));
    return SCW_OK;
}

scw_status sep_eval_slab(scw_sep s, float x0, float y0, float z0, float dx, float dy, float dz, int Nx, int Ny,
                         int k_begin, int k_end, float* dE, int method) {
    scw_ctx ctx = s->ctx;
    SCW_ON_DEVICE(ctx->device);
    // per-kernel timing (scw_ctx_set_timing) times the stages in sequence
    if (s->pipe_chunks > 1 && k_end - k_begin >= kPipeMinPlanes && ctx->sm_count >= 8 && !ctx->timing)
        return sep_eval_slab_pipelined(s, x0, y0, z0, dx, dy, dz, Nx, Ny, k_begin, k_end, dE, method);
    SepEvalPlan p;
    scw_status st = sep_eval_plan_planes(s, x0, y0, z0, dx, dy, dz, Nx, Ny, k_begin, k_end, method, p);
    if (st != SCW_OK) return st;
    if ((st = ctx->sep_scratch.reserve(p.scratch_bytes)) != SCW_OK) return st;
    SCW_CUDA_TRY(cudaEventSynchronize(ctx->desc_done));
    if ((st = ctx->host_desc.reserve(p.desc_bytes)) != SCW_OK) return st;
    if ((st = ctx->desc.reserve(p.desc_bytes)) != SCW_OK) return st;
    sep_eval_desc(p, (char*)ctx->host_desc.ptr);
    SCW_CUDA_TRY(cudaMemcpyAsync(ctx->desc.ptr, ctx->host_desc.ptr, p.desc_bytes, cudaMemcpyHostToDevice, ctx->stream));
    SCW_CUDA_TRY(cudaEventRecord(ctx->desc_done, ctx->stream));
    return sep_eval_record(s, p, (const char*)ctx->desc.ptr, (char*)ctx->sep_scratch.ptr, dE);
}

}  // namespace scw

using scw::fail;

// ------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------
static void sep_free(scw_sep s) {
    if (!s) return;
    ::scw::DeviceScope dev_scope_(s->ctx ? s->ctx->device : -1);
    if (s->dQ && s->own_Q) cudaFree(s->dQ);
    if (s->dKz) cudaFree(s->dKz);
    if (s->dExt) cudaFree(s->dExt);
    if (s->dkx) cudaFree(s->dkx);
    if (s->dky) cudaFree(s->dky);
    if (s->dzb) cudaFree(s->dzb);
    if (s->dBeta) cudaFree(s->dBeta);
    if (s->dslab) cudaFree(s->dslab);
    for (cudaEvent_t e : s->events) cudaEventDestroy(e);
    for (cudaEvent_t e : s->pevents) cudaEventDestroy(e);
    if (s->hi_stream) cudaStreamDestroy(s->hi_stream);
    if (s->up_stream) cudaStreamDestroy(s->up_stream);
    if (s->down_stream) cudaStreamDestroy(s->down_stream);
    delete s;
}

static scw_status sep_create(scw_ctx ctx, int M0, int M1, int n_slices, int modes_per_half, const double* kx,
                             const double* ky, const double* z_boundaries, int halves, scw_sep* out) {
    if (!ctx || !out || M0 <= 0 || M1 <= 0 || n_slices < 0 || modes_per_half < 0 || !kx || !ky || !z_boundaries)
        return fail(SCW_ERR_ARG, "scw_sep_create: bad arguments");
    *out = nullptr;
    SCW_ON_DEVICE(ctx->device);
    scw_sep s = new (std::nothrow) scw_sep_s();
    if (!s) return fail(SCW_ERR_NOMEM, "host allocation");
    s->ctx = ctx;
    s->M0 = M0;
    s->M1 = M1;
    s->MF = M0 * M1;
    s->Z = n_slices;
    s->J = modes_per_half;
    s->Jp = modes_per_half + (modes_per_half & 1);
    s->halves = halves;
    s->kx.assign(kx, kx + M0);
    s->ky.assign(ky, ky + M1);
    s->zb.assign(z_boundaries, z_boundaries + n_slices + 1);
    s->z_layers.resize(n_slices + 1);
    for (int l = 0; l <= n_slices; l++) s->z_layers[l] = (float)z_boundaries[l];
    const size_t nQ = (size_t)n_slices * halves * 3 * s->MF * (size_t)s->Jp;
    bool ok = cudaMalloc(&s->dkx, M0 * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&s->dky, M1 * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&s->dzb, (n_slices + 1) * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&s->dExt, 12 * (size_t)s->MF * sizeof(double2)) == cudaSuccess &&
              cudaMalloc(&s->dKz, ((size_t)n_slices * 2 * s->Jp + 1) * sizeof(double2)) == cudaSuccess;
    if (ok && nQ) {
        ok = cudaMalloc(&s->dQ, nQ * sizeof(float2)) == cudaSuccess;
        s->own_Q = true;
    }
    const size_t nB = (size_t)n_slices * 2 * s->Jp + 1;
    if (ok && halves == 1) ok = cudaMalloc(&s->dBeta, nB * sizeof(double2)) == cudaSuccess;
    if (!ok) {
        sep_free(s);
        return fail(SCW_ERR_NOMEM, "cudaMalloc of the separable coefficient set");
    }
    cudaMemcpy(s->dkx, kx, M0 * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(s->dky, ky, M1 * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(s->dzb, z_boundaries, (n_slices + 1) * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemset(s->dExt, 0, 12 * (size_t)s->MF * sizeof(double2));
    if (nQ) cudaMemset(s->dQ, 0, nQ * sizeof(float2));
    cudaMemset(s->dKz, 0, ((size_t)n_slices * 2 * s->Jp + 1) * sizeof(double2));
    if (s->dBeta) cudaMemset(s->dBeta, 0, nB * sizeof(double2));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        sep_free(s);
        return fail(SCW_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = s;
    return SCW_OK;
}

extern "C" {

scw_status scw_sep_create(scw_ctx ctx, int M0, int M1, int n_slices, int modes_per_half, const double* kx,
                          const double* ky, const double* z_boundaries, scw_sep* out) {
    return sep_create(ctx, M0, M1, n_slices, modes_per_half, kx, ky, z_boundaries, 2, out);
}

scw_status scw_sep_create_paired(scw_ctx ctx, int M0, int M1, int n_slices, int modes_per_half, const double* kx,
                                 const double* ky, const double* z_boundaries, scw_sep* out) {
    return sep_create(ctx, M0, M1, n_slices, modes_per_half, kx, ky, z_boundaries, 1, out);
}

scw_status scw_sep_form(scw_sep s, int* halves) {
    if (!s || !halves) return fail(SCW_ERR_ARG, "scw_sep_form: null argument");
    *halves = s->halves;
    return SCW_OK;
}

scw_status scw_sep_destroy(scw_sep s) {
    sep_free(s);
    return SCW_OK;
}

scw_status scw_sep_set_exterior(scw_sep s, const double* inc, const double* kz_inc, const double* refl,
                                const double* kz_refl, const double* trans, const double* kz_trans) {
    if (!s || !inc || !kz_inc || !refl || !kz_refl || !trans || !kz_trans)
        return fail(SCW_ERR_ARG, "scw_sep_set_exterior: null argument");
    const size_t MF = (size_t)s->MF;
    std::vector<double> h(24 * MF);
    std::memcpy(h.data(), inc, 6 * MF * 8);
    std::memcpy(h.data() + 6 * MF, refl, 6 * MF * 8);
    std::memcpy(h.data() + 12 * MF, trans, 6 * MF * 8);
    std::memcpy(h.data() + 18 * MF, kz_inc, 2 * MF * 8);
    std::memcpy(h.data() + 20 * MF, kz_refl, 2 * MF * 8);
    std::memcpy(h.data() + 22 * MF, kz_trans, 2 * MF * 8);
    SCW_ON_DEVICE(s->ctx->device);
    SCW_CUDA_TRY(cudaMemcpy(s->dExt, h.data(), 24 * MF * 8, cudaMemcpyHostToDevice));
    return SCW_OK;
}

static scw_status upload_kz(scw_sep s, int l, const double* kz_dn, const double* kz_up) {
    const size_t J = (size_t)s->J, Jp = (size_t)s->Jp;
    std::vector<double> kz(4 * Jp, 0.0);
    std::memcpy(kz.data(), kz_dn, 2 * J * 8);
    std::memcpy(kz.data() + 2 * Jp, kz_up, 2 * J * 8);
    SCW_CUDA_TRY(cudaMemcpy(s->dKz + (size_t)l * 2 * Jp, kz.data(), 4 * Jp * 8, cudaMemcpyHostToDevice));
    return SCW_OK;
}

// copies a [3][MF][J] complex64 block into the [3][MF][Jp] device slot (pitched when J is odd)
static scw_status upload_q(scw_sep s, int l, int half, const void* src, cudaMemcpyKind kind, bool async) {
    const size_t J = (size_t)s->J, Jp = (size_t)s->Jp, MF = (size_t)s->MF;
    float2* dst = s->dQ + ((size_t)l * 2 + half) * 3 * MF * Jp;
    if (J == Jp) {
        if (async)
            SCW_CUDA_TRY(cudaMemcpyAsync(dst, src, 3 * MF * J * sizeof(float2), kind, s->ctx->stream));
        else
            SCW_CUDA_TRY(cudaMemcpy(dst, src, 3 * MF * J * sizeof(float2), kind));
    } else {
        if (async)
            SCW_CUDA_TRY(cudaMemcpy2DAsync(dst, Jp * sizeof(float2), src, J * sizeof(float2), J * sizeof(float2),
                                           3 * MF, kind, s->ctx->stream));
        else
            SCW_CUDA_TRY(cudaMemcpy2D(dst, Jp * sizeof(float2), src, J * sizeof(float2), J * sizeof(float2), 3 * MF,
                                      kind));
    }
    return SCW_OK;
}

scw_status scw_sep_set_slice(scw_sep s, int l, const double* kz_dn, const double* Q_dn, const double* kz_up,
                             const double* Q_up) {
    if (!s || l < 0 || l >= s->Z) return fail(SCW_ERR_ARG, "scw_sep_set_slice: slice out of range");
    if (s->halves != 2) return fail(SCW_ERR_STATE, "scw_sep_set_slice: a paired set takes scw_sep_set_slice_paired");
    const size_t J = (size_t)s->J, MF = (size_t)s->MF;
    if (J == 0) return SCW_OK;
    if (!kz_dn || !Q_dn || !kz_up || !Q_up) return fail(SCW_ERR_ARG, "scw_sep_set_slice: null argument");
    SCW_ON_DEVICE(s->ctx->device);
    scw_status st = upload_kz(s, l, kz_dn, kz_up);
    if (st != SCW_OK) return st;
    std::vector<float2> q(3 * MF * J);
    for (int half = 0; half < 2; half++) {
        const double* src = half == 0 ? Q_dn : Q_up;
        for (size_t i = 0; i < 3 * MF * J; i++) q[i] = make_float2((float)src[2 * i], (float)src[2 * i + 1]);
        if ((st = upload_q(s, l, half, q.data(), cudaMemcpyHostToDevice, false)) != SCW_OK) return st;
    }
    return SCW_OK;
}

scw_status scw_sep_set_slice_device(scw_sep s, int l, const double* kz_dn, const void* Q_dn_c64, const double* kz_up,
                                    const void* Q_up_c64) {
    if (!s || l < 0 || l >= s->Z) return fail(SCW_ERR_ARG, "scw_sep_set_slice_device: slice out of range");
    if (s->halves != 2)
        return fail(SCW_ERR_STATE, "scw_sep_set_slice_device: a paired set takes scw_sep_set_slice_paired");
    if (s->J == 0) return SCW_OK;
    if (!kz_dn || !Q_dn_c64 || !kz_up || !Q_up_c64) return fail(SCW_ERR_ARG, "scw_sep_set_slice_device: null argument");
    SCW_ON_DEVICE(s->ctx->device);
    scw_status st = upload_kz(s, l, kz_dn, kz_up);
    if (st != SCW_OK) return st;
    if ((st = upload_q(s, l, 0, Q_dn_c64, cudaMemcpyDefault, true)) != SCW_OK) return st;
    return upload_q(s, l, 1, Q_up_c64, cudaMemcpyDefault, true);
}

scw_status scw_sep_set_slice_paired(scw_sep s, int l, const double* kz_dn, const double* kz_up, const void* V_c64,
                                    const double* beta_dn, const double* beta_up) {
    if (!s || l < 0 || l >= s->Z) return fail(SCW_ERR_ARG, "scw_sep_set_slice_paired: slice out of range");
    if (s->halves != 1) return fail(SCW_ERR_STATE, "scw_sep_set_slice_paired: not a paired set");
    if (s->J == 0) return SCW_OK;
    if (!kz_dn || !kz_up || !V_c64 || !beta_dn || !beta_up)
        return fail(SCW_ERR_ARG, "scw_sep_set_slice_paired: null argument");
    SCW_ON_DEVICE(s->ctx->device);
    scw_status st = upload_kz(s, l, kz_dn, kz_up);
    if (st != SCW_OK) return st;
    const size_t J = (size_t)s->J, Jp = (size_t)s->Jp, MF = (size_t)s->MF;
    std::vector<double> b(4 * Jp, 0.0);
    std::memcpy(b.data(), beta_dn, 2 * J * 8);
    std::memcpy(b.data() + 2 * Jp, beta_up, 2 * J * 8);
    SCW_CUDA_TRY(cudaMemcpy(s->dBeta + (size_t)l * 2 * Jp, b.data(), 4 * Jp * 8, cudaMemcpyHostToDevice));
    float2* dst = s->dQ + (size_t)l * 3 * MF * Jp;
    if (J == Jp)
        SCW_CUDA_TRY(cudaMemcpyAsync(dst, V_c64, 3 * MF * J * sizeof(float2), cudaMemcpyDefault, s->ctx->stream));
    else
        SCW_CUDA_TRY(cudaMemcpy2DAsync(dst, Jp * sizeof(float2), V_c64, J * sizeof(float2), J * sizeof(float2), 3 * MF,
                                       cudaMemcpyDefault, s->ctx->stream));
    return SCW_OK;
}

scw_status scw_sep_set_region_rule(scw_sep s, int rule) {
    if (!s || (rule != 0 && rule != 1)) return fail(SCW_ERR_ARG, "region rule must be 0 or 1");
    s->rule = rule;
    return SCW_OK;
}

scw_status scw_sep_eval_volume_device(scw_sep s, float x_start, float y_start, float z_start, float dx, float dy,
                                      float dz, int Nx, int Ny, int Nz, float* dE, int method) {
    if (!s || !dE || Nx <= 0 || Ny <= 0 || Nz <= 0) return fail(SCW_ERR_ARG, "scw_sep_eval_volume_device: bad arguments");
    return scw::sep_eval(s, 0, x_start, y_start, z_start, dx, dy, dz, Nx, Ny, Nz, dE, method);
}

scw_status scw_sep_eval_volume_host(scw_sep s, const void* Q_host, float x_start, float y_start, float z_start,
                                    float dx, float dy, float dz, int Nx, int Ny, int Nz, float* E_host, int method) {
    if (!s || !E_host || Nx <= 0 || Ny <= 0 || Nz <= 0 || (s->J > 0 && !Q_host))
        return fail(SCW_ERR_ARG, "scw_sep_eval_volume_host: bad arguments");
    return scw::sep_eval_volume_host(s, (const float2*)Q_host, x_start, y_start, z_start, dx, dy, dz, Nx, Ny, 0, Nz,
                                     E_host, method);
}

scw_status scw_sep_eval_slab_host(scw_sep s, const void* Q_host, float x_start, float y_start, float z_start, float dx,
                                  float dy, float dz, int Nx, int Ny, int k_begin, int k_end, float* E_host,
                                  int method) {
    if (!s || !E_host || Nx <= 0 || Ny <= 0 || k_begin < 0 || k_end <= k_begin || (s->J > 0 && !Q_host))
        return fail(SCW_ERR_ARG, "scw_sep_eval_slab_host: bad arguments");
    return scw::sep_eval_volume_host(s, (const float2*)Q_host, x_start, y_start, z_start, dx, dy, dz, Nx, Ny, k_begin,
                                     k_end, E_host, method);
}

scw_status scw_sep_eval_slab_device(scw_sep s, float x_start, float y_start, float z_start, float dx, float dy,
                                    float dz, int Nx, int Ny, int k_begin, int k_end, float* dE, int method) {
    if (!s || !dE || Nx <= 0 || Ny <= 0 || k_begin < 0 || k_end <= k_begin)
        return fail(SCW_ERR_ARG, "scw_sep_eval_slab_device: bad arguments");
    return scw::sep_eval_slab(s, x_start, y_start, z_start, dx, dy, dz, Nx, Ny, k_begin, k_end, dE, method);
}

scw_status scw_sep_set_streaming(scw_sep s, int64_t chunk_bytes, int64_t slab_bytes) {
    if (!s || chunk_bytes < 0 || slab_bytes < 0) return fail(SCW_ERR_ARG, "scw_sep_set_streaming: bad arguments");
    s->chunk_bytes = (size_t)chunk_bytes;
    s->slab_target = (size_t)slab_bytes;
    return SCW_OK;
}

scw_status scw_sep_set_pipeline(scw_sep s, int chunks, int synth_sm_div) {
    if (!s || chunks < 0 || chunks > 64 || synth_sm_div < 1 || synth_sm_div > 16)
        return fail(SCW_ERR_ARG, "scw_sep_set_pipeline: bad arguments");
    s->pipe_chunks = chunks;
    s->pipe_synth_div = synth_sm_div;
    return SCW_OK;
}

scw_status scw_sep_set_tiles(scw_sep s, int ctr_shape) {
    if (!s || ctr_shape < 0 || ctr_shape > 1) return fail(SCW_ERR_ARG, "scw_sep_set_tiles: bad arguments");
    s->ctr_shape = ctr_shape;
    return SCW_OK;
}

scw_status scw_sep_eval_plane_device(scw_sep s, int axis, float a_start, float b_start, float c, float d, int N,
                                     float* dE, int method) {
    if (!s || !dE || N <= 0 || axis < 0 || axis > 2) return fail(SCW_ERR_ARG, "scw_sep_eval_plane_device: bad arguments");
    if (axis == 0) return scw::sep_eval(s, 0, a_start, b_start, c, d, d, 0.f, N, N, 1, dE, method);
    if (axis == 2) return scw::sep_eval(s, 1, a_start, b_start, c, d, d, 0.f, N, N, 1, dE, method);
    return scw::sep_eval(s, 2, a_start, b_start, c, d, d, 0.f, N, N, 1, dE, method);
}

scw_status scw_sep_gpu_cw_evaluate(scw_sep s, float* E_xy, float* E_xz, float* E_yz, float x_start, float y_start,
                                   float z_start, float x, float y, float z, float d, int N, int device, int method) {
    if (!s || !E_xy || !E_xz || !E_yz || N <= 0) return fail(SCW_ERR_ARG, "scw_sep_gpu_cw_evaluate: bad arguments");
    scw_ctx ctx = s->ctx;
    if (device != ctx->device) return fail(SCW_ERR_ARG, "scw_sep_gpu_cw_evaluate: device differs from the set's device");
    SCW_ON_DEVICE(ctx->device);
    const size_t plane = (size_t)N * N * 6;
    scw_status st = ctx->planes_out.reserve(3 * plane * sizeof(float));
    if (st != SCW_OK) return st;
    float* d0 = (float*)ctx->planes_out.ptr;
    if ((st = scw_sep_eval_plane_device(s, 0, x_start, y_start, z, d, N, d0, method)) != SCW_OK) return st;
    if ((st = scw_sep_eval_plane_device(s, 2, x_start, z_start, y, d, N, d0 + plane, method)) != SCW_OK) return st;
    if ((st = scw_sep_eval_plane_device(s, 1, y_start, z_start, x, d, N, d0 + 2 * plane, method)) != SCW_OK) return st;
    SCW_CUDA_TRY(cudaMemcpyAsync(E_xy, d0, plane * 4, cudaMemcpyDeviceToHost, ctx->stream));
    SCW_CUDA_TRY(cudaMemcpyAsync(E_xz, d0 + plane, plane * 4, cudaMemcpyDeviceToHost, ctx->stream));
    SCW_CUDA_TRY(cudaMemcpyAsync(E_yz, d0 + 2 * plane, plane * 4, cudaMemcpyDeviceToHost, ctx->stream));
    return scw_ctx_synchronize(ctx);
}

}  // extern "C"
