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
// Pipeline (one CTA per SM, persistent over the row tiles of one 128-column x tile), warp
// specialised with mbarrier hand-offs:
//   warps 0-7   epilogue: warp w reads TMEM lane quarter w % 4 (32 x-values) for the tile's
//               rows 8 (w / 4) .. 8 (w / 4) + 7 -> registers -> global (accumulator full/empty)
//   warps 8-14  producers: build B (hi, lo) of the next tile into one of two shared buffers,
//               writing whole 16-byte core rows in address order (no bank conflicts)
//   warp 15     one thread issues the MMAs into one of two TMEM accumulators and commits them
// A (hi, lo), the x-phase table of the CTA's x tile, is written once into tensor memory by warps
// 0-3 (lane x = row x, one 32-bit column per tf32 element or per pair of bf16 elements, at
// columns 256 and 256 + K columns) and read from there by every MMA, so the tensor core's operand
// reads from shared memory are B's alone.  TMEM columns: accumulators at 0 and 128 (96 each),
// A hi / lo above 256.  B uses the SWIZZLE_NONE K-major canonical layout in shared memory:
// 8-row x 16-byte core matrices stored contiguously, LBO = 128 B between core matrices along K,
// SBO = (K bytes / 16) * 128 B between 8-row groups.
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
constexpr uint32_t kTmemCols = 512;     // the whole TMEM (1 CTA / SM)
// TMEM layout for kXS x tiles per CTA: the two accumulators at columns 0 and acc_col(kXS), then the
// A tables from a_col(kXS): x tile t's hi at a_col + 2 t acols, its lo acols further
__host__ __device__ constexpr uint32_t acc_col(int xs) { return xs == 1 ? 128u : 96u; }
__host__ __device__ constexpr uint32_t a_col(int xs) { return xs == 1 ? 256u : 192u; }
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

// the same with A read from tensor memory at a_tmem (lanes 0..M-1, K along the columns)
template <int kKind>
__device__ __forceinline__ void umma_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    if (kKind == 0) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
            "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(acc)
            : "memory");
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
            "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(acc)
            : "memory");
    }
}

// this warp's 32 lanes x 8 consecutive columns of 32-bit values
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&v)[8]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
                 "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
                 : "memory");
}
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 lanes x 16 consecutive columns of 32-bit values
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* v) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
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

// round-to-nearest-even to the 10-bit tf32 mantissa with integer operations (keeps the split
// off the conversion pipe); finite inputs only, which is all the operands ever are
__device__ __forceinline__ float tf32_rn(float x) {
    const uint32_t b = __float_as_uint(x);
    return __uint_as_float((b + 0xFFFu + ((b >> 13) & 1u)) & 0xFFFFE000u);
}

__device__ __forceinline__ __nv_bfloat16 bf16_rn(float x) {
    const uint32_t b = __float_as_uint(x);
    return __ushort_as_bfloat16((unsigned short)((b + 0x7FFFu + ((b >> 16) & 1u)) >> 16));
}

template <int kKind>
struct Split;

template <>
struct Split<0> {           // tf32 in fp32 containers
    using T = float;
    static constexpr int kBytes = 4;
    // hi: x with the low 13 mantissa bits cleared; lo = x - hi is exact, and the tensor core
    // reads its top 19 bits, so x = hi + lo to within 2^-20 |x|
    __device__ static void split(float x, float& hi, float& lo) {
        hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
        lo = x - hi;
    }
};

template <>
struct Split<1> {           // bf16
    using T = __nv_bfloat16;
    static constexpr int kBytes = 2;
    __device__ static void split(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
        hi = bf16_rn(x);
        lo = bf16_rn(x - __bfloat162float(hi));
    }
};

// bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned) from shared to global
// memory, tracked by this thread's bulk groups
__device__ __forceinline__ void bulk_store(void* gdst, const void* ssrc, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(smem_u32(ssrc)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// this thread's committed bulk copies have finished reading shared memory
__device__ __forceinline__ void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// ... and have finished writing global memory
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// one 32-bit TMEM column: a tf32 element, or two bf16 elements (the first in the low half)
template <int kKind>
__device__ __forceinline__ uint32_t pack1(const typename Split<kKind>::T* v);

template <>
__device__ __forceinline__ uint32_t pack1<0>(const float* v) { return __float_as_uint(v[0]); }

template <>
__device__ __forceinline__ uint32_t pack1<1>(const __nv_bfloat16* v) {
    return (uint32_t)__bfloat16_as_ushort(v[0]) | ((uint32_t)__bfloat16_as_ushort(v[1]) << 16);
}

// the negated values of a packed core row: a sign flip per tf32 element or per bf16 half
template <int kKind>
__device__ __forceinline__ uint4 neg4(uint4 v) {
    const uint32_t s = kKind == 0 ? 0x80000000u : 0x80008000u;
    return make_uint4(v.x ^ s, v.y ^ s, v.z ^ s, v.w ^ s);
}

template <int kKind>
__device__ __forceinline__ uint4 pack4(const typename Split<kKind>::T* v);

template <>
__device__ __forceinline__ uint4 pack4<0>(const float* v) {        // 4 tf32 values
    return make_uint4(__float_as_uint(v[0]), __float_as_uint(v[1]), __float_as_uint(v[2]), __float_as_uint(v[3]));
}

template <>
__device__ __forceinline__ uint4 pack4<1>(const __nv_bfloat16* v) { // 8 bf16 values
    uint4 r;
    r.x = (uint32_t)__bfloat16_as_ushort(v[0]) | ((uint32_t)__bfloat16_as_ushort(v[1]) << 16);
    r.y = (uint32_t)__bfloat16_as_ushort(v[2]) | ((uint32_t)__bfloat16_as_ushort(v[3]) << 16);
    r.z = (uint32_t)__bfloat16_as_ushort(v[4]) | ((uint32_t)__bfloat16_as_ushort(v[5]) << 16);
    r.w = (uint32_t)__bfloat16_as_ushort(v[6]) | ((uint32_t)__bfloat16_as_ushort(v[7]) << 16);
    return r;
}

constexpr int kEpiWarps = 8, kProdWarps = 7;      // 16 warps with the MMA warp: 128 registers each
constexpr int kEpiRows = kRows * 4 / kEpiWarps;     // output rows per epilogue warp and tile (8)
constexpr int kTStages = 3;                          // staged T tiles in flight (cp.async ring)
constexpr int kMaxKH = 12;                           // fast producer path: 16-byte core columns per K half

// Staged T rows (float2) in shared memory.  Fast path (Mk a multiple of the elements per core
// row): a row holds a multiple of 8 16-byte chunks and chunk c of row r sits at c ^ t_swz(r), so
// the producers' 16-byte reads (8 lanes per phase: 4 consecutive rows x 2 consecutive tasks
// along K) land on 8 distinct bank groups.  Generic path: rows of Mk, unswizzled.
__host__ __device__ constexpr bool t_fast(int Mk, int kind) { return Mk % (kind == 0 ? 4 : 8) == 0 && Mk % 2 == 0; }
__host__ __device__ constexpr int t_row_stride(int Mk, int kind) { return t_fast(Mk, kind) ? ((Mk / 2 + 7) / 8) * 16 : Mk; }
template <int kKind>
__device__ __forceinline__ int t_swz(int row) { return kKind == 0 ? ((row & 1) | ((row & 2) << 1)) : (row & 3); }

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem_dst)), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// OR of v over the producer warps (named barrier 1): keeps their loop decisions uniform so
// every producer thread reaches the same named barriers
__device__ __forceinline__ int producers_any(int v) {
    int r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.s32 q, %1, 0;\n\t"
        "bar.red.or.pred p, 1, %2, q;\n\tselp.s32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"(v), "n"(kProdWarps * 32)
        : "memory");
    return r;
}
// named barrier 2 + part among the 4 epilogue warps of a half-tile; the vote form returns the OR
// of v over them, so their loop decisions stay uniform
__device__ __forceinline__ void epi_part_sync(int part) {
    asm volatile("bar.sync %0, 128;" ::"r"(2 + part) : "memory");
}
__device__ __forceinline__ int epi_part_any(int v, int part) {
    int r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.s32 q, %1, 0;\n\t"
        "bar.red.or.pred p, %2, 128, q;\n\tselp.s32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"(v), "r"(2 + part)
        : "memory");
    return r;
}
constexpr int kWsThreads = (kEpiWarps + kProdWarps + 1) * 32;

// kXS x tiles of 128 columns per CTA: the B operand of a row tile, built once by the producers,
// serves kXS MMA groups (one per x tile, each into its own accumulator), so the producers' work per
// output byte falls by kXS.  Work unit u = i kXS + t (row tile i, x tile t) uses accumulator u & 1.
template <int kKind, int kXS>
__global__ void __launch_bounds__(kWsThreads, 1)
synth_tc_kernel(const float2* __restrict__ T, const float2* __restrict__ F, int nrows, int ncols, int Mk, int Kp,
                int srows, float* __restrict__ out, int* __restrict__ err) {
    using E = typename Split<kKind>::T;
    constexpr int EB = Split<kKind>::kBytes;
    constexpr int EPC = 16 / EB;                              // elements per 16-byte core row
    extern __shared__ __align__(1024) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t kbytes = (uint32_t)Kp * EB;
    const int KC = (int)(kbytes / 16);                        // 16-byte core columns along K
    const uint32_t sbo = (uint32_t)KC * 128;
    const uint32_t b_bytes = (kN / 8) * sbo;
    const uint32_t acols = kbytes / 4;                        // TMEM columns of A (hi or lo): K * EB / 4
    unsigned char* sB0 = smem;                                // slot s, part h: sB0 + (2 s + h) b_bytes
    // ring of kTStages staged T tiles [kRows * 3][tstr], filled by cp.async kTStages - 1 tiles ahead
    const int t_slot = (((kRows * 3 * t_row_stride(Mk, kKind) * 8 + 127) / 128) * 128) / 8;   // float2 per slot
    float2* sT = reinterpret_cast<float2*>(sB0 + 4 * b_bytes);
    const int t_tile = kRows * 3 * Mk;                           // float2 of T per tile
    // fast producer path: Mk a multiple of the elements per core row, swizzled T rows
    const bool fast = t_fast(Mk, kKind);
    const int tstr = t_row_stride(Mk, kKind);
    // output staging: srows rows of 32 x-values x 6 floats (768 bytes) per epilogue warp
    float* sOut = reinterpret_cast<float*>(sT + kTStages * t_slot);
    uint64_t* bar = reinterpret_cast<uint64_t*>(sOut + kEpiWarps * srows * 192);
    uint64_t* full_b = bar;          // [2] producers -> MMA
    uint64_t* empty_b = bar + 2;     // [2] MMA completion -> producers
    uint64_t* acc_full = bar + 4;    // [2] MMA completion -> epilogue
    uint64_t* acc_empty = bar + 6;   // [2] epilogue -> MMA
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 8);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(bar + 9);

    const int x0 = blockIdx.x * kM * kXS;
    constexpr uint32_t kAccCol = acc_col(kXS), kACol = a_col(kXS);
    const int ntiles = (nrows + kRows - 1) / kRows;
    const int n_my = blockIdx.y < ntiles ? (ntiles - 1 - (int)blockIdx.y) / (int)gridDim.y + 1 : 0;

    for (uint32_t o = tid * 16; o < 4 * b_bytes; o += kWsThreads * 16)
        *reinterpret_cast<uint4*>(smem + o) = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        for (int i = 0; i < 2; i++) {
            mbar_init(&full_b[i], kProdWarps * 32);     // every producer thread arrives after its fence
            mbar_init(&empty_b[i], 1);
            mbar_init(&acc_full[i], 1);
            mbar_init(&acc_empty[i], kEpiWarps * 32);   // every epilogue thread arrives after its TMEM reads
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, kTmemCols);
        tmem_relinquish();
    }
    __syncthreads();
    const uint32_t tmem = *tmem_slot;
    // A: the phase tables of the CTA's x tiles into TMEM, lane x = x0 + 128 t + 32 w + lane (warps
    // 0-3), 8 columns per store: tf32 one element per column, bf16 elements 2c (low half) and 2c + 1
    // per column c
    if (warp < 4) {
      for (int xt = 0; xt < kXS; xt++) {
        const int xg = x0 + xt * kM + warp * 32 + lane;
        const uint32_t acol = kACol + 2u * (uint32_t)xt * acols;
        constexpr int EPW = 4 / EB;                           // elements per 32-bit column
        for (uint32_t c0 = 0; c0 < acols; c0 += 8) {
            uint32_t vh[8], vl[8];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                E hi[EPW], lo[EPW];
#pragma unroll
                for (int e = 0; e < EPW; e++) {
                    const int k = ((int)c0 + i) * EPW + e;
                    float v = 0.f;
                    if (xg < ncols && k < 2 * Mk) {
                        const float2 f = F[(long long)(k < Mk ? k : k - Mk) * ncols + xg];
                        v = k < Mk ? f.x : f.y;
                    }
                    Split<kKind>::split(v, hi[e], lo[e]);
                }
                vh[i] = pack1<kKind>(hi);
                vl[i] = pack1<kKind>(lo);
            }
            const uint32_t lanes = (uint32_t)(warp * 32) << 16;
            tmem_st8(tmem + lanes + acol + c0, vh);
            tmem_st8(tmem + lanes + acol + acols + c0, vl);
        }
      }
        tmem_st_wait();
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    if (warp >= kEpiWarps && warp < kEpiWarps + kProdWarps) {
        // ---------------- producers ----------------
        const int pt = tid - kEpiWarps * 32;                  // 0 .. kProdWarps * 32 - 1
        const int n4 = t_tile / 2;
        // fast path: tile ti's rows of T into ring slot ti % kTStages with 16-byte cp.async
        // (row (r, c) at slot + (3 r + c) * tstr, chunks swizzled; the buffer has slack past the
        // last row, whose values are masked below), one commit group per tile, empty groups past
        // the last tile
        // row = e / h as (e * hinv) >> 20 with hinv = ceil(2^20 / h): exact for e < 2^11 (n4 = 24 Mk
        // <= 1920 chunks) and h < 2^9, and it keeps the division off the per-tile copy loop
        const int h = Mk / 2;                                      // float4 per T row
        const uint32_t hinv = fast ? ((1u << 20) + (uint32_t)h - 1u) / (uint32_t)h : 0u;
        auto issue_t = [&](int ti) {
            if (ti < n_my) {
                const int rr0 = ((int)blockIdx.y + ti * (int)gridDim.y) * kRows;
                const float4* src = reinterpret_cast<const float4*>(T + (long long)rr0 * 3 * Mk);
                float2* dst = sT + (ti % kTStages) * t_slot;
                for (int e = pt; e < n4; e += kProdWarps * 32) {
                    const int row = (int)(((uint32_t)e * hinv) >> 20);
                    cp_async16(reinterpret_cast<float4*>(dst + row * tstr) + ((e - row * h) ^ t_swz<kKind>(row)),
                               src + e);
                }
            }
            cp_async_commit();
        };
        // fast path (K has no padding: KC = 2 KH core columns, the second half holding the same T
        // values as the first): task = (8-row block nb, row pair nq, core column kh of the first
        // half); lanes: nq fastest, then kh. One task reads 16 bytes x EPC/2 of T row (4 nb + nq)
        // once, splits its Re and Im parts into hi and lo once, and writes the Re (n even) and Im
        // (n odd) rows of B in both halves: core column kh gets [Re T, Im T], core column kh + KH
        // gets [-Im T, Re T] (negation is a sign flip of the split parts, exact). A task's offsets
        // are the same for every tile, so they are computed once: t_off[u] = T offset in float2 of
        // the slot (-1: no task), the first of the task's EPC/2 chunks once swizzled; b_off[u] = B
        // byte offset of core column kh | T row / 3 << 20 | (order of the task's chunks, XOR) << 24
        // | (kh odd) << 28.  The host admits the fast path for KH <= kMaxKH only.
        constexpr int kTasks = (kN / 8 * kMaxKH * 4 + kProdWarps * 32 - 1) / (kProdWarps * 32);
        const int KH = KC / 2;
        int t_off[kTasks];
        uint32_t b_off[kTasks];
#pragma unroll
        for (int u = 0; u < kTasks; u++) {
            const int tsk = pt + u * kProdWarps * 32;
            const int q = tsk >> 2, nq = tsk & 3;
            const int nb = q / KH, kh = q - nb * KH;
            const int trow = 4 * nb + nq, k0 = kh * EPC;
            const bool live = tsk < (kN / 8) * KH * 4 && k0 < Mk;
            constexpr int m = EPC / 2 - 1;                        // chunks of one task - 1
            const int g = t_swz<kKind>(trow);
            const int c0 = k0 / 2;                                // first chunk of the task in its row
            t_off[u] = live ? trow * tstr + 2 * (c0 ^ (g & ~m)) : -1;
            b_off[u] = ((uint32_t)nb * sbo + (uint32_t)kh * 128u + (uint32_t)(2 * nq) * 16u) |
                       ((uint32_t)(trow / 3) << 20) | ((uint32_t)(g & m) << 24) | ((uint32_t)(kh & 1) << 28);
        }
        const uint32_t half_off = (uint32_t)KH * 128u;             // core column kh -> kh + KH
        if (fast)
            for (int ti = 0; ti < kTStages - 1; ti++) issue_t(ti);
        // one producer barrier per tile: it publishes tile i's T (this thread's copies are in once
        // all but the newest group have completed), frees the slot of tile i - 1 for the copies of
        // tile i + kTStages - 1 issued after it, and makes the abort decision uniform
        for (int i = 0; i < n_my; i++) {
            const int s = i & 1;
            int stop = *abort_flag;
            if (!stop && i >= 2 && !mbar_wait(&empty_b[s], (uint32_t)(((i >> 1) - 1) & 1))) stop = 1;
            const int r0 = ((int)blockIdx.y + i * (int)gridDim.y) * kRows;
            unsigned char* bh = sB0 + (2 * s + 0) * b_bytes;
            unsigned char* bl = sB0 + (2 * s + 1) * b_bytes;
            float2* sTi = sT + (i % kTStages) * t_slot;
            if (fast) {
                cp_async_wait<kTStages - 2>();
            } else if (!stop) {
                for (int e = pt; e < t_tile; e += kProdWarps * 32) sTi[e] = T[(long long)r0 * 3 * Mk + e];
            }
            if (producers_any(stop)) {
                *abort_flag = 1;
                break;
            }
            if (fast) issue_t(i + kTStages - 1);
            if (fast) {
                // loads of all of this thread's tasks issued before any use; rows past nrows
                // (the last tile) read as zeros
                const int rows_left = nrows - r0;
                float4 tv[kTasks][EPC / 2];
#pragma unroll
                for (int u = 0; u < kTasks; u++) {
                    const bool ok = t_off[u] >= 0 && (int)((b_off[u] >> 20) & 15u) < rows_left;
                    const float4* tp = reinterpret_cast<const float4*>(sTi + (ok ? t_off[u] : 0));
                    const int gx = (int)((b_off[u] >> 24) & 3u);
#pragma unroll
                    for (int e2 = 0; e2 < EPC / 2; e2++) tv[u][e2] = ok ? tp[e2 ^ gx] : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < kTasks; u++) {
                    if (t_off[u] < 0) continue;
                    E rh[EPC], rl[EPC], ih[EPC], il[EPC];         // hi / lo of Re T and Im T
#pragma unroll
                    for (int e2 = 0; e2 < EPC / 2; e2++) {
                        const float4 t = tv[u][e2];              // (Re, Im) of two T values
                        Split<kKind>::split(t.x, rh[2 * e2], rl[2 * e2]);
                        Split<kKind>::split(t.z, rh[2 * e2 + 1], rl[2 * e2 + 1]);
                        Split<kKind>::split(t.y, ih[2 * e2], il[2 * e2]);
                        Split<kKind>::split(t.w, ih[2 * e2 + 1], il[2 * e2 + 1]);
                    }
                    const uint4 vrh = pack4<kKind>(rh), vrl = pack4<kKind>(rl);
                    const uint4 vih = pack4<kKind>(ih), vil = pack4<kKind>(il);
                    const uint4 nih = neg4<kKind>(vih), nil = neg4<kKind>(vil);
                    const uint32_t b1 = b_off[u] & 0xFFFFFu, b2 = b1 + half_off;
                    // s = 0 (Re E): [Re T | -Im T];  s = 1 (Im E): [Im T | Re T].  The store order
                    // alternates with kh so each warp store covers all 8 bank groups
                    if (((b_off[u] >> 28) & 1u) == 0) {
                        *reinterpret_cast<uint4*>(bh + b1) = vrh;
                        *reinterpret_cast<uint4*>(bh + b1 + 16) = vih;
                        *reinterpret_cast<uint4*>(bl + b1) = vrl;
                        *reinterpret_cast<uint4*>(bl + b1 + 16) = vil;
                        *reinterpret_cast<uint4*>(bh + b2) = nih;
                        *reinterpret_cast<uint4*>(bh + b2 + 16) = vrh;
                        *reinterpret_cast<uint4*>(bl + b2) = nil;
                        *reinterpret_cast<uint4*>(bl + b2 + 16) = vrl;
                    } else {
                        *reinterpret_cast<uint4*>(bh + b1 + 16) = vih;
                        *reinterpret_cast<uint4*>(bh + b1) = vrh;
                        *reinterpret_cast<uint4*>(bl + b1 + 16) = vil;
                        *reinterpret_cast<uint4*>(bl + b1) = vrl;
                        *reinterpret_cast<uint4*>(bh + b2 + 16) = vrh;
                        *reinterpret_cast<uint4*>(bh + b2) = nih;
                        *reinterpret_cast<uint4*>(bl + b2 + 16) = vrl;
                        *reinterpret_cast<uint4*>(bl + b2) = nil;
                    }
                }
            } else {
                // generic path: one 16-byte core row per group, groups in address order
                int q = pt >> 3;
                int nb = q / KC, kc = q - nb * KC;
                const int nlo = pt & 7;
                constexpr int kStepQ = kProdWarps * 32 / 8;
                for (int g = pt; g < kN * KC; g += kProdWarps * 32) {
                    const int n = (nb << 3) | nlo;
                    const int r = n / 6, c = (n - 6 * r) >> 1, sri = n & 1;
                    const bool live = (r0 + r) < nrows;
                    const float2* trow = sTi + (r * 3 + c) * tstr;
                    E hi[EPC], lo[EPC];
#pragma unroll
                    for (int e = 0; e < EPC; e++) {
                        const int k = kc * EPC + e;
                        float v = 0.f;
                        if (live && k < 2 * Mk) {
                            const bool first = k < Mk;
                            const float2 t = trow[first ? k : k - Mk];
                            v = sri == 0 ? (first ? t.x : -t.y) : (first ? t.y : t.x);
                        }
                        Split<kKind>::split(v, hi[e], lo[e]);
                    }
                    *reinterpret_cast<uint4*>(bh + (uint32_t)g * 16) = pack4<kKind>(hi);
                    *reinterpret_cast<uint4*>(bl + (uint32_t)g * 16) = pack4<kKind>(lo);
                    kc += kStepQ;
                    while (kc >= KC) {
                        kc -= KC;
                        nb++;
                    }
                }
            }
            fence_proxy_async();
            mbar_arrive(&full_b[s]);
        }
        cp_async_wait<0>();        // no copy into shared memory outlives the loop (also after an abort)
    } else if (warp == kEpiWarps + kProdWarps) {
        // ---------------- MMA issuer ----------------
        const uint32_t ab_fmt = kKind == 0 ? 2u : 1u;
        const uint32_t idesc = (1u << 4) | (ab_fmt << 7) | (ab_fmt << 10) | ((uint32_t)(kN >> 3) << 17) |
                               ((uint32_t)(kM >> 4) << 24);
        const int nksteps = (int)(kbytes / 32);
        int issued = 0;
        if (lane == 0) {
            bool stop = false;
            for (int i = 0; i < n_my && !stop; i++) {
                if (*abort_flag) break;
                const int s = i & 1;
                if (!mbar_wait(&full_b[s], (uint32_t)((i >> 1) & 1))) {
                    *abort_flag = 1;
                    break;
                }
                const uint32_t b_hi = smem_u32(sB0 + (2 * s) * b_bytes), b_lo = smem_u32(sB0 + (2 * s + 1) * b_bytes);
                for (int xt = 0; xt < kXS; xt++) {
                    const int u = i * kXS + xt, a = u & 1;
                    if (u >= 2 && !mbar_wait(&acc_empty[a], (uint32_t)(((u >> 1) - 1) & 1))) {
                        *abort_flag = 1;
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d = tmem + (uint32_t)a * kAccCol;
                    const uint32_t a_hi = tmem + kACol + 2u * (uint32_t)xt * acols, a_lo = a_hi + acols;
                    for (int ks = 0; ks < nksteps; ks++) {
                        const uint32_t ko = (uint32_t)ks * 256u;    // 32 bytes of K = two 16-byte core columns of B
                        const uint32_t ka = (uint32_t)ks * 8u;      // the same 32 bytes of K = 8 TMEM columns of A
                        umma_ta<kKind>(d, a_hi + ka, make_desc(b_hi + ko, 128, sbo), idesc, ks > 0);
                        umma_ta<kKind>(d, a_hi + ka, make_desc(b_lo + ko, 128, sbo), idesc, 1);
                        umma_ta<kKind>(d, a_lo + ka, make_desc(b_hi + ko, 128, sbo), idesc, 1);
                    }
                    umma_commit(&acc_full[a]);
                    issued = u + 1;
                }
                if (!stop) umma_commit(&empty_b[s]);      // B slot s is free once this row tile's MMAs are done
            }
            // the accumulators must be idle before TMEM is freed: wait for the last commit
            if (issued > 0) mbar_wait(&acc_full[(issued - 1) & 1], (uint32_t)(((issued - 1) >> 1) & 1));
        }
        __syncwarp();
    } else {
        // -------- epilogue (warp w: TMEM lanes 32 (w % 4) .. + 31, rows kEpiRows (w / 4) ..) --------
        // TMEM -> registers (8 rows x 6 floats per lane); the accumulator is released as soon as the
        // values are in registers.  The four warps of a half-tile (part) then stage their 32 x-values
        // of each row side by side (warp q at float offset 192 q, lane l at 6 l), so that a row of
        // the tile is 3 KB contiguous in shared memory as in global memory, and one thread of the
        // part hands each row to the bulk copy engine (cp.async.bulk shared -> global): 16 copies of
        // 3 KB per tile.  Tiles whose rows are ragged or not 16-byte aligned are stored by the warps'
        // lanes.  The part's warps synchronise on named barrier 2 + part (128 threads); the abort
        // decision is taken by a vote on that barrier, so all four reach the same barriers.
        const int quarter = warp & 3, part = warp >> 2;
        const bool issuer = quarter == 0 && lane == 0;
        float* stage = sOut + part * srows * (kM * 6);
        const bool aligned = (ncols & 1) == 0 && (reinterpret_cast<uintptr_t>(out) & 15u) == 0;
        for (int u = 0; u < n_my * kXS; u++) {
            const int a = u & 1, i = u / kXS;
            const int xs = x0 + (u - i * kXS) * kM;           // first x of this unit's x tile
            const int xw = xs + quarter * 32;                 // first x of this warp
            const int nx = min(32, ncols - xw);              // valid x of this warp
            // every row of a whole, aligned x tile goes out as one 3 KB copy
            const bool bulk = xs + kM <= ncols && aligned;
            int stop = *abort_flag;
            if (!stop && !__all_sync(0xffffffffu, mbar_wait(&acc_full[a], (uint32_t)((u >> 1) & 1)))) stop = 1;
            if (epi_part_any(stop, part)) {
                *abort_flag = 1;
                break;
            }
            tc_fence_after();
            const int r0 = ((int)blockIdx.y + i * (int)gridDim.y) * kRows + part * kEpiRows;
            const uint32_t tbase =
                tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)a * kAccCol + (uint32_t)(part * kEpiRows * 6);
            uint32_t v[kEpiRows * 6];
#pragma unroll
            for (int c16 = 0; c16 < kEpiRows * 6 / 16; c16++) tmem_ld16(tbase + (uint32_t)(16 * c16), &v[16 * c16]);
            tmem_ld_wait();
            tc_fence_before();
            mbar_arrive(&acc_empty[a]);
            for (int g0 = 0; g0 < kEpiRows; g0 += srows) {
                // the staging rows are reusable once the part's earlier bulk copies have read them
                if (issuer) bulk_wait_read0();
                epi_part_sync(part);
#pragma unroll
                for (int r = 0; r < kEpiRows; r++) {
                    if (r < g0 || r >= g0 + srows) continue;
                    float2* st = reinterpret_cast<float2*>(stage + (r - g0) * (kM * 6) + quarter * 192);
                    st[3 * lane + 0] = make_float2(__uint_as_float(v[6 * r + 0]), __uint_as_float(v[6 * r + 1]));
                    st[3 * lane + 1] = make_float2(__uint_as_float(v[6 * r + 2]), __uint_as_float(v[6 * r + 3]));
                    st[3 * lane + 2] = make_float2(__uint_as_float(v[6 * r + 4]), __uint_as_float(v[6 * r + 5]));
                }
                fence_proxy_async();              // the staged rows visible to the bulk copies
                epi_part_sync(part);
                if (bulk) {
                    if (issuer) {
                        for (int r = g0; r < g0 + srows && r0 + r < nrows; r++)
                            bulk_store(out + ((long long)(r0 + r) * ncols + xs) * 6, stage + (r - g0) * (kM * 6),
                                       (uint32_t)(kM * 6 * sizeof(float)));
                        bulk_commit();
                    }
                } else {
                    for (int r = g0; r < g0 + srows; r++) {
                        const int row = r0 + r;
                        if (row >= nrows || nx <= 0) break;       // warp-uniform
                        float* dst = out + ((long long)row * ncols + xw) * 6;
                        const float* src = stage + (r - g0) * (kM * 6) + quarter * 192;
                        for (int f = lane; f < nx * 6; f += 32) dst[f] = src[f];
                    }
                }
            }
        }
        // every bulk copy of this part has written global memory before the kernel ends
        if (issuer) bulk_wait_all();
        __syncwarp();
    }
    __syncthreads();
    if (tid == 0 && *abort_flag) atomicExch(err, 1);
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
    const size_t t_tile_bytes = ((size_t)tc::kRows * 3 * tc::t_row_stride(Mk, kind) * 8 + 127) / 128 * 128;
    // output staging rows per epilogue warp: 8 (one bulk group per tile) when shared memory allows
    const size_t fixed = (tc::kN / 8) * sbo * 4 + tc::kTStages * t_tile_bytes + 128;
    int srows = tc::kEpiRows;
    while (srows > 1 && fixed + (size_t)tc::kEpiWarps * srows * 768 > 227 * 1024) srows /= 2;
    const size_t smem = fixed + (size_t)tc::kEpiWarps * srows * 768;
    if (smem > 227 * 1024) return SCW_ERR_UNSUPPORTED;
    const size_t acols = (size_t)Kp * EB / 4;                 // TMEM columns of one A table (hi or lo)
    if (tc::a_col(1) + 2 * acols > tc::kTmemCols) return SCW_ERR_UNSUPPORTED;   // A (hi, lo) in TMEM
    // two x tiles per CTA (B shared) where both A tables fit beside the accumulators and the grid
    // has more than one x tile
    const int xs = (tc::a_col(2) + 4 * acols <= tc::kTmemCols && ncols > tc::kM) ? 2 : 1;
    // the fast producer path covers at most kMaxKH 16-byte core columns per K half
    if (tc::t_fast(Mk, kind) && (size_t)Kp * EB / 32 > (size_t)tc::kMaxKH) return SCW_ERR_UNSUPPORTED;
    if (!ctx->tc_err) {
        if (cudaMalloc(&ctx->tc_err, sizeof(int)) != cudaSuccess) return fail(SCW_ERR_NOMEM, "cudaMalloc error flag");
    }
    // cleared once per synchronisation: a flag raised by an earlier launch stays raised
    if (!ctx->tc_pending_check) SCW_CUDA_TRY(cudaMemsetAsync(ctx->tc_err, 0, sizeof(int), ctx->stream));
    const int xt = (ncols + tc::kM * xs - 1) / (tc::kM * xs);
    const int ntiles = (nrows + tc::kRows - 1) / tc::kRows;
    int yt = std::max(1, (ctx->synth_ctas > 0 ? ctx->synth_ctas : ctx->sm_count) / xt);
    yt = std::min(yt, ntiles);
    dim3 grid(xt, yt);
    LaunchTimer lt(ctx, kind == 0 ? "synth_tc_kernel<tf32x3>" : "synth_tc_kernel<bf16x3>");
    auto launch = [&](auto kernel) -> scw_status {
        SCW_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kernel<<<grid, tc::kWsThreads, smem, ctx->stream>>>(T, F, nrows, ncols, Mk, Kp, srows, out, ctx->tc_err);
        return SCW_OK;
    };
    scw_status ls;
    if (kind == 0) ls = xs == 2 ? launch(tc::synth_tc_kernel<0, 2>) : launch(tc::synth_tc_kernel<0, 1>);
    else ls = xs == 2 ? launch(tc::synth_tc_kernel<1, 2>) : launch(tc::synth_tc_kernel<1, 1>);
    if (ls != SCW_OK) return ls;
    SCW_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    ctx->tc_pending_check = true;
    return SCW_OK;
}

}  // namespace scw
