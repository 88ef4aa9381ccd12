// Tensor-core output GEMM of the separable evaluator (tcgen05 / TMEM, sm_103a).
//
//   E_c(row, x) = sum_m F(m, x) T_c(row, m)        (complex; F = e^{i k_m x}, T from stage 2a)
//
// as a real GEMM D = A . B^T with the real embedding of the complex product:
//   A[x][k]  (M = 128 x-values per tile, K = 2 Mk padded to a multiple of 8 / 16):
//            A[x][m] = Re F(m, x),   A[x][Mk + m] = Im F(m, x)
//   B[n][k]  (N = 16 rows x 3 components x re/im = 96, n = 6 r + 2 c + s):
//            s = 0: B[n][m] = Re T,  B[n][Mk + m] = -Im T      -> D = Re E
//            s = 1: B[n][m] = Im T,  B[n][Mk + m] =  Re T      -> D = Im E
// so TMEM lane x holds, for each of the tile's 16 rows, the 6 floats of E(row, x) in output
// order and the epilogue writes 24 contiguous bytes per (row, x): lanes of a warp cover 32
// consecutive x, i.e. 768 contiguous bytes per row (coalesced).
//
// Precision: each operand is split into a hi and a lo part (TF32: round-to-nearest tf32 hi,
// lo = tf32(x - hi); BF16: bf16 hi, bf16 lo) and D = Ahi.Bhi + Ahi.Blo + Alo.Bhi, FP32
// accumulation in TMEM.
//
// Pipeline (one CTA per SM, 128 threads, persistent over row tiles of one 128-column x tile):
// A (hi, lo) is built once in shared memory; per row tile all threads build B (hi, lo) in one
// of two shared buffers, thread 0 issues the MMAs into one of two TMEM accumulators and
// commits them to an mbarrier, and the epilogue of the previous tile (all 4 warps, one TMEM
// lane quarter each) runs while the tensor cores work.  Operands use the SWIZZLE_NONE
// K-major canonical layout: 8-row x 16-byte core matrices stored contiguously, LBO = 128 B
// between core matrices along K, SBO = (K bytes / 16) * 128 B between 8-row groups.
// Every mbarrier wait is bounded; on timeout the kernel records an error, waits (bounded)
// for its own MMAs, frees its TMEM and returns, and the host reports SCW_ERR_TIMEOUT.
#include <cuda_bf16.h>
#include <algorithm>
#include <cstdint>

#include "scw_sep.h"

namespace scw {

namespace tc {

constexpr int kM = 128;          // x-values per tile (TMEM lanes)
constexpr int kRows = 16;        // output rows per tile
constexpr int kN = kRows * 6;    // 96 accumulator columns per tile
constexpr int kThreads = 128;
constexpr uint32_t kTmemCols = 512;     // two 96-column accumulators at columns 0 and 128; whole TMEM (1 CTA / SM)
constexpr long long kSpinLimit = 1ll << 22;   // polls per mbarrier wait before giving up

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait; false if the limit was reached
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (long long i = 0; i < kSpinLimit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

template <int kKind>   // 0: tf32, 1: f16-kind (bf16 operands)
__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    if (kKind == 0) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
            : "memory");
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
            : "memory");
    }
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 lanes x 32 consecutive columns of 32-bit values
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// SWIZZLE_NONE K-major shared-memory matrix descriptor (sm_100 format, version bits 46-48 = 1)
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// element (row, k) of a K-major SWIZZLE_NONE operand with 16-byte core rows
__device__ __forceinline__ uint32_t core_offset(int row, int kbyte, uint32_t sbo) {
    return (uint32_t)(row >> 3) * sbo + (uint32_t)(kbyte >> 4) * 128u + (uint32_t)(row & 7) * 16u + (uint32_t)(kbyte & 15);
}

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

template <int kKind>
struct Split;

template <>
struct Split<0> {           // tf32 in fp32 containers
    using T = float;
    static constexpr int kBytes = 4;
    __device__ static void split(float x, float& hi, float& lo) {
        hi = tf32_rna(x);
        lo = tf32_rna(x - hi);
    }
};

template <>
struct Split<1> {           // bf16
    using T = __nv_bfloat16;
    static constexpr int kBytes = 2;
    __device__ static void split(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
        hi = __float2bfloat16_rn(x);
        lo = __float2bfloat16_rn(x - __bfloat162float(hi));
    }
};

template <int kKind>
__global__ void __launch_bounds__(kThreads, 1)
synth_tc_kernel(const float2* __restrict__ T, const float2* __restrict__ F, int nrows, int ncols, int Mk, int Kp,
                float* __restrict__ out, int* __restrict__ err) {
    using E = typename Split<kKind>::T;
    constexpr int EB = Split<kKind>::kBytes;
    extern __shared__ __align__(1024) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t kbytes = (uint32_t)Kp * EB;              // bytes of K per row
    const uint32_t sbo = (kbytes / 16) * 128;               // 8-row group stride
    const uint32_t a_bytes = (kM / 8) * sbo;
    const uint32_t b_bytes = (kN / 8) * sbo;
    unsigned char* sA_hi = smem;
    unsigned char* sA_lo = sA_hi + a_bytes;
    unsigned char* sB[2][2] = {{sA_lo + a_bytes, sA_lo + a_bytes + b_bytes},
                               {sA_lo + a_bytes + 2 * b_bytes, sA_lo + a_bytes + 3 * b_bytes}};   // [slot][hi/lo]
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sA_lo + a_bytes + 4 * b_bytes);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + 2);

    const int x0 = blockIdx.x * kM;
    const int ntiles = (nrows + kRows - 1) / kRows;

    // zero all operand memory (covers the K padding and out-of-range rows / columns)
    for (uint32_t o = tid * 16; o < 2 * a_bytes + 4 * b_bytes; o += kThreads * 16)
        *reinterpret_cast<uint4*>(smem + o) = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, kTmemCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // A: the phase table of this x tile
    for (int e = tid; e < kM * Mk; e += kThreads) {
        const int x = e / Mk, m = e % Mk;
        const int xg = x0 + x;
        const float2 f = xg < ncols ? F[(long long)m * ncols + xg] : make_float2(0.f, 0.f);
        E rh, rl, ih, il;
        Split<kKind>::split(f.x, rh, rl);
        Split<kKind>::split(f.y, ih, il);
        *reinterpret_cast<E*>(sA_hi + core_offset(x, m * EB, sbo)) = rh;
        *reinterpret_cast<E*>(sA_lo + core_offset(x, m * EB, sbo)) = rl;
        *reinterpret_cast<E*>(sA_hi + core_offset(x, (Mk + m) * EB, sbo)) = ih;
        *reinterpret_cast<E*>(sA_lo + core_offset(x, (Mk + m) * EB, sbo)) = il;
    }

    // instruction descriptor: D f32, A/B tf32 (2) or bf16 (1), both K-major, N = 96, M = 128
    const uint32_t ab_fmt = kKind == 0 ? 2u : 1u;
    const uint32_t idesc = (1u << 4) | (ab_fmt << 7) | (ab_fmt << 10) | ((uint32_t)(kN >> 3) << 17) |
                           ((uint32_t)(kM >> 4) << 24);
    const int kstep_bytes = 32;                               // K per MMA instruction: 32 bytes
    const int nksteps = (int)(kbytes / kstep_bytes);
    bool ok = true;              // CTA-uniform between the barriers of the tile loop
    int issued = 0;              // MMA groups committed (group i: slot i & 1, parity (i >> 1) & 1)
    int waited = 0;              // MMA groups awaited

    // epilogue of the tile whose MMA group index is `grp`
    auto epilogue = [&](int tile, int grp) {
        const int slot = grp & 1;
        bool got = mbar_wait(&mbar[slot], (uint32_t)((grp >> 1) & 1));
        got = __all_sync(0xffffffffu, got);
        waited = grp + 1;
        tc_fence_after();
        if (!got) {
            ok = false;
            return;
        }
        const int r0 = tile * kRows;
        const int xg = x0 + warp * 32 + lane;
        const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(slot * 128);
        uint32_t v[32];
#pragma unroll 1
        for (int q = 0; q < kN / 32; q++) {
            tmem_ld32(tbase + (uint32_t)(q * 32), v);
            tmem_ld_wait();
#pragma unroll
            for (int cc = 0; cc < 32; cc += 2) {
                const int col = q * 32 + cc;          // even column: (row r, component c, re); odd: im
                const int r = col / 6, w = col % 6;
                const int row = r0 + r;
                if (xg < ncols && row < nrows) {
                    const float2 val = make_float2(__uint_as_float(v[cc]), __uint_as_float(v[cc + 1]));
                    *reinterpret_cast<float2*>(out + ((long long)row * ncols + xg) * 6 + w) = val;
                }
            }
        }
        tc_fence_before();
    };

    int prev_tile = -1;
    for (int tile = blockIdx.y; tile < ntiles; tile += gridDim.y) {
        if (!ok) break;
        const int s = issued & 1;
        // B for this tile into buffer s (the MMA group that last read it was awaited by the
        // previous epilogue)
        const int r0 = tile * kRows;
        for (int e = tid; e < kRows * 3 * Mk; e += kThreads) {
            const int r = e / (3 * Mk);
            const int rem = e % (3 * Mk);
            const int c = rem / Mk, m = rem % Mk;
            const int row = r0 + r;
            const float2 tv = row < nrows ? T[((long long)row * 3 + c) * Mk + m] : make_float2(0.f, 0.f);
            E reh, rel, imh, iml, nimh, niml;
            Split<kKind>::split(tv.x, reh, rel);
            Split<kKind>::split(tv.y, imh, iml);
            Split<kKind>::split(-tv.y, nimh, niml);
            const int n_re = r * 6 + c * 2, n_im = n_re + 1;
            unsigned char* bh = sB[s][0];
            unsigned char* bl = sB[s][1];
            *reinterpret_cast<E*>(bh + core_offset(n_re, m * EB, sbo)) = reh;
            *reinterpret_cast<E*>(bl + core_offset(n_re, m * EB, sbo)) = rel;
            *reinterpret_cast<E*>(bh + core_offset(n_re, (Mk + m) * EB, sbo)) = nimh;
            *reinterpret_cast<E*>(bl + core_offset(n_re, (Mk + m) * EB, sbo)) = niml;
            *reinterpret_cast<E*>(bh + core_offset(n_im, m * EB, sbo)) = imh;
            *reinterpret_cast<E*>(bl + core_offset(n_im, m * EB, sbo)) = iml;
            *reinterpret_cast<E*>(bh + core_offset(n_im, (Mk + m) * EB, sbo)) = reh;
            *reinterpret_cast<E*>(bl + core_offset(n_im, (Mk + m) * EB, sbo)) = rel;
        }
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t d = tmem + (uint32_t)(s * 128);
            const uint32_t a_hi = smem_u32(sA_hi), a_lo = smem_u32(sA_lo);
            const uint32_t b_hi = smem_u32(sB[s][0]), b_lo = smem_u32(sB[s][1]);
            for (int ks = 0; ks < nksteps; ks++) {
                const uint32_t ko = (uint32_t)ks * 256u;    // 32 bytes of K = two 16-byte core columns
                umma<kKind>(d, make_desc(a_hi + ko, 128, sbo), make_desc(b_hi + ko, 128, sbo), idesc, ks > 0);
                umma<kKind>(d, make_desc(a_hi + ko, 128, sbo), make_desc(b_lo + ko, 128, sbo), idesc, 1);
                umma<kKind>(d, make_desc(a_lo + ko, 128, sbo), make_desc(b_hi + ko, 128, sbo), idesc, 1);
            }
            umma_commit(&mbar[s]);
        }
        issued++;
        if (prev_tile >= 0) epilogue(prev_tile, issued - 2);
        ok = __syncthreads_and(ok) != 0;
        prev_tile = tile;
    }
    if (prev_tile >= 0 && ok) epilogue(prev_tile, issued - 1);
    ok = __syncthreads_and(ok) != 0;
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        // drain: wait (bounded) for every committed MMA group before freeing TMEM
        for (int g = waited; g < issued; g++) mbar_wait(&mbar[g & 1], (uint32_t)((g >> 1) & 1));
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

}  // namespace tc

scw_status sep_synth_tc(scw_ctx ctx, const float2* T, const float2* F, int nrows, int ncols, int Mk, float* out,
                        int method) {
    const int kind = method == SCW_SEP_TF32X3 ? 0 : 1;
    const int EB = kind == 0 ? 4 : 2;
    const int kalign = kind == 0 ? 8 : 16;                  // K per MMA instruction
    const int Kp = (2 * Mk + kalign - 1) / kalign * kalign;
    const size_t sbo = (size_t)Kp * EB / 16 * 128;
    const size_t smem = (tc::kM / 8) * sbo * 2 + (tc::kN / 8) * sbo * 4 + 64;
    if (smem > 227 * 1024) return SCW_ERR_UNSUPPORTED;
    if (!ctx->tc_err) {
        if (cudaMalloc(&ctx->tc_err, sizeof(int)) != cudaSuccess) return fail(SCW_ERR_NOMEM, "cudaMalloc error flag");
    }
    SCW_CUDA_TRY(cudaMemsetAsync(ctx->tc_err, 0, sizeof(int), ctx->stream));
    const int xt = (ncols + tc::kM - 1) / tc::kM;
    const int ntiles = (nrows + tc::kRows - 1) / tc::kRows;
    int yt = std::max(1, ctx->sm_count / xt);
    yt = std::min(yt, ntiles);
    dim3 grid(xt, yt);
    LaunchTimer lt(ctx, kind == 0 ? "synth_tc_kernel<tf32x3>" : "synth_tc_kernel<bf16x3>");
    if (kind == 0) {
        SCW_CUDA_TRY(cudaFuncSetAttribute(tc::synth_tc_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        tc::synth_tc_kernel<0><<<grid, tc::kThreads, smem, ctx->stream>>>(T, F, nrows, ncols, Mk, Kp, out, ctx->tc_err);
    } else {
        SCW_CUDA_TRY(cudaFuncSetAttribute(tc::synth_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        tc::synth_tc_kernel<1><<<grid, tc::kThreads, smem, ctx->stream>>>(T, F, nrows, ncols, Mk, Kp, out, ctx->tc_err);
    }
    SCW_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    ctx->tc_pending_check = true;
    return SCW_OK;
}

}  // namespace scw
