// kernels_umma.cu -- FP32-accurate GEMM on the 5th-generation tensor cores.
//
//   C[m][n] = sum_k A[m][k] * B[n][k]         (A, B K-contiguous, N <= 512, K % 16 == 0)
//
// FP32 accuracy from TF32 units: every operand x is stored as hi = tf32(x) and lo = tf32(x - hi)
// (split_tf32_kernel), and the tile accumulates hi*hi + hi*lo + lo*hi in FP32.  The dropped lo*lo
// term and the truncation of lo are below 2^-21 of |x*y|, i.e. at FP32 rounding level.  The faster
// tier stores the data operand A once as tf32(x) and accumulates hi*hi + hi*lo (the fixed B keeps
// its split), an error of about 2^-12 of |x*y| per product.
//
// Persistent, warp-specialised CTAs (one per SM) walk the 128 x N output tiles: warp E / lane 0
// streams A and B tiles into shared memory with TMA (cp.async.bulk.tensor, 64-byte swizzle)
// through one mbarrier ring of stages that runs on across tiles; warp E + 1 / lane 0 issues
// tcgen05.mma (M = 128, N = 128 or 256) into one of two N-column TMEM accumulators, releasing each
// stage with tcgen05.commit; the E = kGemmEpiWarps warps read the other accumulator back with
// tcgen05.ld (warp e its 32 TMEM lanes 32 (e % 4) .. = tile rows, every (E / 4)-th chunk of 32
// columns) and store it while the next tile accumulates, then hand it back through an mbarrier.
// Every wait is bounded (globaltimer); on a timeout the kernel sets an error word, waits (bounded)
// for the copies it issued and the MMAs it started, frees its TMEM and returns.
#include "lss_kernels.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

namespace lss {

constexpr int kBM = 128, kBK = 16;
constexpr int kTileA = kBM * kBK * 4;                   // 8 KB
constexpr int kSmemBudget = 196 * 1024;                 // stage buffers per CTA
constexpr uint64_t kWaitNs = 2000000000ull;             // 2 s
constexpr int kGemmEpiWarps = 8;                        // a multiple of 4
constexpr int kGemmThreads = (kGemmEpiWarps + 2) * 32;

// Two uses of one kernel:
//   kPlain     C[m][n] = sum_k A[m][k] B[n][k]; tile N = 256; B rows = n
//   kToeplitz  the circular high-pass: A = channel-major wrapped windows [(b, c)][time], B = a fixed
//              N x K band matrix G[j][k] = taps[k - j] (N = 256 output times per tile for groups of
//              batches, 128 for a few); the tile at output time w0 reads A columns w0 + k, and the
//              epilogue stores Y[b][w0 + j][c] as its tf32 split (hi, lo) or as tf32 alone
enum UmmaMode { kPlain = 0, kToeplitz = 1 };

struct UmmaArgs {
    float* out;       // kPlain: C; kToeplitz: Y (hi)
    float* out_lo;    // kToeplitz: Y (lo)
    int M, N, K;
    int64_t ldc;      // kPlain
    int chans, wlen;  // kToeplitz: C and W of a window (rows of A are (b, c) = (r / chans, r % chans))
    int* err;
    // kPlain, optional: C also stored channel-major, zt[(row / wlen) * N + n][row % wlen] at row
    // pitch zpitch, as its tf32 split (zt_lo null: tf32 alone)
    float* zt_hi;
    float* zt_lo;
    int zpitch;
    int zt_bf16;      // zt as its BF16 split (bf16 arrays)
    const float* col_scale;   // kPlain, optional: C[m][n] *= col_scale[n] (the FP8 operands' scales)
    int slices;       // kPlain: K split this many ways, slice z written to C + z M ldc (1: no split)
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t gtimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false after kWaitNs (the caller records the timeout)
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    if (mbar_try(bar, parity)) return true;
    const uint64_t t0 = gtimer();
    for (;;) {
        if (mbar_try(bar, parity)) return true;
        if (gtimer() - t0 > kWaitNs) return false;
    }
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
        : "memory");
}
// shared-memory matrix descriptor: K-major, 64-byte swizzle, 8-row groups 512 B apart
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);          // start address
    d |= (uint64_t)1u << 16;                          // leading byte offset (unused when swizzled)
    d |= (uint64_t)((512u >> 4) & 0x3FFFu) << 32;     // stride byte offset
    d |= (uint64_t)1u << 46;                          // descriptor version
    d |= (uint64_t)4u << 61;                          // swizzle 64B
    return d;
}
// instruction descriptor: D = F32, A = B = TF32, both K-major, M = 128, N = BN
template <int BN>
struct IdescTf32 {
    static constexpr uint32_t value =
        (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
};

// the same for A = B = BF16 (kind::f16, K = 16 per instruction = the same 32 bytes)
template <int BN>
struct IdescBf16 {
    static constexpr uint32_t value =
        (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
};

template <int BN>
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(IdescBf16<BN>::value), "r"(accumulate)
        : "memory");
}

// the same for A = B = FP8 e4m3 (kind::f8f6f4, K = 32 per instruction = the same 32 bytes)
template <int BN>
struct IdescE4m3 {
    static constexpr uint32_t value =
        (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
};

template <int BN>
__device__ __forceinline__ void mma_e4m3(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(IdescE4m3<BN>::value), "r"(accumulate)
        : "memory");
}

template <int BN>
__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(IdescTf32<BN>::value), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// ALO = false: A is TF32 data without a remainder (the two products hi_a*hi_b + hi_a*lo_b; the
// fixed B operand keeps its split), for the tensor-core tier whose activations are stored once.
// BF16: the operands are BF16 splits (hi = bf16(x), lo = bf16(x - hi)) multiplied by kind::f16
// MMAs: a K-step is 32 elements, still 64-byte rows, so tiles, swizzle and pipeline are unchanged.
// LOWP: one product of the operands' hi parts only -- 1 = BF16 (kind::f16), 2 = FP8 e4m3
// (kind::f8f6f4, a K-step of 64 elements); only hi tiles are loaded, so a stage is half the bytes
// and twice the stages fit.  The epilogue then scales column n by args.col_scale[n] when given.
template <int BN, int MODE, bool ALO, bool BF16 = false, int LOWP = 0>
__global__ void __launch_bounds__(kGemmThreads, 1)
umma_gemm_3xtf32(const __grid_constant__ CUtensorMap tA_hi, const __grid_constant__ CUtensorMap tA_lo,
                 const __grid_constant__ CUtensorMap tB_hi, const __grid_constant__ CUtensorMap tB_lo, UmmaArgs args) {
    constexpr int kBN = BN;
    // two accumulators at columns 0 and kBN; the allocation is a power of two (256 or 512)
    constexpr int kTmemCols = 2 * kBN <= 256 ? 256 : 512;
    constexpr int kKE = LOWP == 2 ? 4 * kBK : (BF16 ? 2 * kBK : kBK);   // elements per K-step (64 bytes of each row)
    constexpr int kTileB = kBN * kBK * 4;
    constexpr int kStageBytes = LOWP ? kTileA + kTileB : 2 * kTileA + 2 * kTileB;
    constexpr int kLoadBytes = LOWP ? kStageBytes : (ALO ? kStageBytes : kTileA + 2 * kTileB);   // bytes the TMA lands per stage
    constexpr int kStages = kSmemBudget / kStageBytes;
    const int M = args.M, N = args.N, K = args.K, S = args.slices;
    int* err = args.err;
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages], tfull_bar[2], tempty_bar[2], drain_bar;
    __shared__ uint32_t tmem_base_s;
    __shared__ int abort_raw;
    volatile int& abort_s = abort_raw;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nk = K / kKE;
    const int tiles_n = (N + kBN - 1) / kBN, tiles_m = (M + kBM - 1) / kBM;
    const int ntiles = tiles_n * tiles_m * S;
    // tile t: output columns n0 = (t % tiles_n) kBN, rows m0 = ((t / tiles_n) % tiles_m) kBM, K slice
    // z = t / (tiles_n tiles_m) -- the column tiles of one row block run on neighbouring CTAs and
    // share its A tiles through L2.  Split K (S > 1, plain mode): slice z multiplies the K-steps
    // [nk z / S, nk (z + 1) / S) and writes its partial tile to output slice z (the caller sums them).
    auto tile_of = [&](int t, int& n0, int& m0, int& kt0, int& nkl) {
        const int z = t / (tiles_n * tiles_m), r = t - z * tiles_n * tiles_m;
        n0 = (r % tiles_n) * kBN;
        m0 = (r / tiles_n) * kBM;
        kt0 = (int)((int64_t)nk * z / S);
        nkl = (int)((int64_t)nk * (z + 1) / S) - kt0;
        return z;
    };
    // 1024-byte aligned stage buffers: [A_hi][A_lo][B_hi][B_lo] per stage
    const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
    // (LOWP: [A_hi][B_hi] per stage)
    auto sA_hi = [&](int s) { return base + (uint32_t)(s * kStageBytes); };
    auto sA_lo = [&](int s) { return base + (uint32_t)(s * kStageBytes + kTileA); };
    auto sB_hi = [&](int s) { return base + (uint32_t)(s * kStageBytes + (LOWP ? 1 : 2) * kTileA); };
    auto sB_lo = [&](int s) { return base + (uint32_t)(s * kStageBytes + 2 * kTileA + kTileB); };

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(smem_u32(&full_bar[s]), 1);
            mbar_init(smem_u32(&empty_bar[s]), 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(smem_u32(&tfull_bar[a]), 1);
            mbar_init(smem_u32(&tempty_bar[a]), kGemmEpiWarps);   // one arrival per epilogue warp
        }
        mbar_init(smem_u32(&drain_bar), 1);
        abort_s = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_s;

    if (warp == kGemmEpiWarps && lane == 0) {
        // ---- producer: TMA, one ring of stages across all tiles of this CTA ----
        int q = 0;
        bool stop = false;
        for (int tile = blockIdx.x; tile < ntiles && !stop; tile += gridDim.x) {
            int n0, m0, kt0, nkl;
            tile_of(tile, n0, m0, kt0, nkl);
            for (int kt = 0; kt < nkl; ++kt, ++q) {
                const int s = q % kStages;
                const uint32_t round = (uint32_t)(q / kStages);
                if (!mbar_wait(smem_u32(&empty_bar[s]), (round & 1u) ^ 1u) || abort_s) {
                    atomicOr(err, 1);
                    abort_s = 1;
                    stop = true;
                    break;
                }
                const uint32_t fb = smem_u32(&full_bar[s]);
                mbar_expect_tx(fb, kLoadBytes);
                const int k0 = (kt0 + kt) * kKE;   // a multiple of 64 bytes
                // Toeplitz: A columns start at the tile's output time n0 (a multiple of 128), B is the
                // same band matrix for every tile
                const int ax = (MODE == kToeplitz) ? n0 + k0 : k0;
                const int by = (MODE == kToeplitz) ? 0 : n0;
                tma_load_2d(sA_hi(s), &tA_hi, fb, ax, m0);
                if constexpr (ALO && !LOWP) tma_load_2d(sA_lo(s), &tA_lo, fb, ax, m0);
                tma_load_2d(sB_hi(s), &tB_hi, fb, k0, by);
                if constexpr (!LOWP) tma_load_2d(sB_lo(s), &tB_lo, fb, k0, by);
            }
        }
        // the copies of the last rounds must have landed before the CTA may exit
        for (int kt = (q > kStages ? q - kStages : 0); kt < q; ++kt)
            if (!mbar_wait(smem_u32(&full_bar[kt % kStages]), (uint32_t)(kt / kStages) & 1u)) atomicOr(err, 4);
    } else if (warp == kGemmEpiWarps + 1 && lane == 0) {
        // ---- MMA issuer: tile i accumulates into TMEM columns (i % 2) kBN ----
        int q = 0, i = 0;
        for (int tile = blockIdx.x; tile < ntiles && !abort_s; tile += gridDim.x, ++i) {
            const int ab = i & 1;
            if (!mbar_wait(smem_u32(&tempty_bar[ab]), ((uint32_t)(i >> 1) & 1u) ^ 1u) || abort_s) {
                atomicOr(err, 2);
                abort_s = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t d = tmem + (uint32_t)(ab * kBN);
            int n0, m0, kt0, nkl;
            tile_of(tile, n0, m0, kt0, nkl);
            bool stop = false;
            for (int kt = 0; kt < nkl; ++kt, ++q) {
                const int s = q % kStages;
                const uint32_t round = (uint32_t)(q / kStages);
                if (!mbar_wait(smem_u32(&full_bar[s]), round & 1u) || abort_s) {
                    atomicOr(err, 2);
                    abort_s = 1;
                    stop = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
                for (int kk = 0; kk < 2; ++kk) {          // 32 bytes (8 tf32 / 16 bf16 / 32 e4m3) per MMA
                    const uint32_t off = (uint32_t)kk * 32u;
                    const uint64_t ah = smem_desc(sA_hi(s) + off), al = smem_desc(sA_lo(s) + off);
                    const uint64_t bh = smem_desc(sB_hi(s) + off), bl = smem_desc(sB_lo(s) + off);
                    const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
                    if constexpr (LOWP == 1) {
                        mma_bf16<BN>(d, ah, bh, acc);
                    } else if constexpr (LOWP == 2) {
                        mma_e4m3<BN>(d, ah, bh, acc);
                    } else if constexpr (BF16) {
                        mma_bf16<BN>(d, ah, bh, acc);
                        mma_bf16<BN>(d, ah, bl, 1u);
                        if constexpr (ALO) mma_bf16<BN>(d, al, bh, 1u);
                    } else {
                        mma_tf32<BN>(d, ah, bh, acc);
                        mma_tf32<BN>(d, ah, bl, 1u);
                        if constexpr (ALO) mma_tf32<BN>(d, al, bh, 1u);
                    }
                }
                mma_commit(smem_u32(&empty_bar[s]));        // frees the stage once these MMAs finish
            }
            if (stop) break;
            mma_commit(smem_u32(&tfull_bar[ab]));           // the accumulator is complete
        }
        // every MMA issued has finished before the TMEM is released
        mma_commit(smem_u32(&drain_bar));
        if (!mbar_wait(smem_u32(&drain_bar), 0u)) atomicOr(err, 2);
    } else if (warp < kGemmEpiWarps) {
        // ---- epilogue: TMEM -> registers -> global, overlapping the next tile's MMAs ----
        // warp e reads TMEM lanes 32 (e % 4) .. + 31 (its tile rows), column chunks e / 4, e / 4 +
        // kGemmEpiWarps / 4, ... of 32
        const int quad = warp & 3;
        int i = 0;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
            const int ab = i & 1;
            // one decision per warp: the tcgen05.ld below is .sync.aligned
            const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&tfull_bar[ab]), (uint32_t)(i >> 1) & 1u) && !abort_s);
            if (!ok) {
                if (lane == 0) atomicOr(err, 8);
                abort_s = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            int n0, m0, kt0, nkl;
            const int z = tile_of(tile, n0, m0, kt0, nkl);
            const int row = m0 + quad * 32 + lane;
            for (int c0 = 32 * (warp >> 2); c0 < kBN && n0 + c0 < N; c0 += 32 * (kGemmEpiWarps / 4)) {
                uint32_t r[32];
                const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(ab * kBN + c0);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
                    "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
                      "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                      "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                    : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if constexpr (MODE == kToeplitz) {
                    // row = (b, c); column j = output time n0 + c0 + j; lanes = consecutive channels
                    if (row < M) {
                        const int b = row / args.chans, c = row - b * args.chans;
                        for (int j = 0; j < 32; ++j) {
                            const int w = n0 + c0 + j;
                            if (w < args.wlen) {
                                const float v = __uint_as_float(r[j]);
                                const int64_t o = ((int64_t)b * args.wlen + w) * args.chans + c;
                                if constexpr (BF16) {
                                    // the BF16 split, for the next GEMM on the BF16 tier
                                    const __nv_bfloat16 h = __float2bfloat16_rn(v);
                                    reinterpret_cast<__nv_bfloat16*>(args.out)[o] = h;
                                    reinterpret_cast<__nv_bfloat16*>(args.out_lo)[o] =
                                        __float2bfloat16_rn(v - __bfloat162float(h));
                                } else {
                                    uint32_t h;
                                    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
                                    args.out[o] = __uint_as_float(h);
                                    if (args.out_lo) args.out_lo[o] = v - __uint_as_float(h);
                                }
                            }
                        }
                    }
                    continue;
                }
                if (row < M) {
                    // (out null: only the channel-major copy is wanted)
                    float* crow = args.out ? args.out + ((int64_t)z * M + row) * args.ldc + n0 + c0 : nullptr;
                    const int ncol = min(32, N - (n0 + c0));
                    if (args.col_scale) {
#pragma unroll
                        for (int j = 0; j < 32; ++j)
                            if (j < ncol) r[j] = __float_as_uint(__uint_as_float(r[j]) * __ldg(args.col_scale + n0 + c0 + j));
                    }
                    if (args.zt_hi) {
                        // lanes hold consecutive rows = consecutive times of one channel row of zt
                        const int b = row / args.wlen, w = row - b * args.wlen;
                        const int64_t o = ((int64_t)b * N + n0 + c0) * args.zpitch + w;
#pragma unroll
                        for (int j = 0; j < 32; ++j) {
                            if (j < ncol) {
                                const float v = __uint_as_float(r[j]);
                                const int64_t oj = o + (int64_t)j * args.zpitch;
                                if (args.zt_bf16) {
                                    const __nv_bfloat16 h = __float2bfloat16_rn(v);
                                    reinterpret_cast<__nv_bfloat16*>(args.zt_hi)[oj] = h;
                                    reinterpret_cast<__nv_bfloat16*>(args.zt_lo)[oj] =
                                        __float2bfloat16_rn(v - __bfloat162float(h));
                                } else {
                                    uint32_t h;
                                    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
                                    args.zt_hi[oj] = __uint_as_float(h);
                                    if (args.zt_lo) args.zt_lo[oj] = v - __uint_as_float(h);
                                }
                            }
                        }
                    }
                    if (!crow) {
                    } else if (ncol == 32 && ((((uintptr_t)crow) & 15) == 0)) {
#pragma unroll
                        for (int j = 0; j < 32; j += 4)
                            *reinterpret_cast<float4*>(crow + j) = make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]),
                                                                               __uint_as_float(r[j + 2]), __uint_as_float(r[j + 3]));
                    } else {
#pragma unroll
                        for (int j = 0; j < 32; ++j)
                            if (j < ncol) crow[j] = __uint_as_float(r[j]);
                    }
                }
            }
            // the accumulator may be overwritten once every epilogue warp has read it
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&tempty_bar[ab]));
        }
    }
    __syncwarp();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// hi = tf32(x) (round to nearest, ties away), lo = x - hi (exact in fp32)
__global__ void split_tf32_kernel(const float* __restrict__ x, float* __restrict__ hi, float* __restrict__ lo,
                                  int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = x[i];
        uint32_t h;
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
        const float hf = __uint_as_float(h);
        hi[i] = hf;
        lo[i] = v - hf;
    }
}

// ------------------------------------------------------------------------------------------
// temporal basis convolution as a band GEMM over all components of a group at once:
//   Bpc[b][w][k][c] = sum_m wPCA[k][m] * Z[b][w + m - nt/2][c]
// A = the channel-major whitened windows Zt[(b, c)][time] (M = 128 (b, c) rows per tile).  A tile
// covers TW output times w0..w0+TW-1 of the kg components of its group and the ks K-steps of input
// times from x0 = w0 - hr on.  B of K-step s stacks the components' band matrices along N:
// B_s[g TW + j][i] = wPCA[cg kg + g][step s + i - j - d] (d = hr - nt/2), one resident tile per
// K-step, so a K-step is one MMA of N = kg TW per product (three on the split operands) instead of
// one narrow MMA per component: the tile count per unit of output, not the math, bounded the
// narrow form.  Out-of-window input times (< 0 or >= W) come from the TMA zero fill.
//
// Persistent CTAs (one per SM), warp-specialised: CTA b serves component group b % ncg; warp E /
// lane 0 loads its group's bands once, then A tiles through a kConvStages mbarrier ring; warp
// E + 1 / lane 0 issues tcgen05.mma (M = 128, N = ng TW) into one of two TMEM accumulators of
// kg TW columns; the E = kConvEpiWarps warps 0..E-1 drain the other accumulator into Bpc while the
// next tile accumulates -- warp e reads TMEM lanes 32 (e % 4) .. + 31 (its (b, c) rows), column
// chunks of 32 (one component's 32 output times) e / 4, e / 4 + E / 4, ...  The CTAs of different
// groups walk the same (rows, times) blocks in step and share their A tiles through L2.  Bounded
// waits as in the GEMM above.
// ------------------------------------------------------------------------------------------
constexpr int kConvStages = 4;
constexpr int kConvEpiWarps = 8;                        // a multiple of 4
constexpr int kConvThreads = (kConvEpiWarps + 2) * 32;
constexpr int kConvMaxK = 8;
constexpr int kConvSmemMax = 220 * 1024;

struct ConvArgs {
    float* out_hi;
    float* out_lo;
    int nrows;      // nb * C
    int chans, wlen;
    int kc;         // components
    int ks, hr, tw; // ConvGeometry
    int kg, ncg;    // components per group, groups
    int ntiles_w;
    int* err;
};

// instruction descriptors with N chosen at run time (N % 16 == 0, 16 <= N <= 256)
__device__ __forceinline__ uint32_t idesc_n(uint32_t kind_bits, int n) {
    return kind_bits | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16_rt(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_tf32_rt(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// one chunk of the epilogue: element j (output time wh + j) of this lane's (b, c) row goes to
// o0 + j step.  OUT: 0 = fp32, 1 = tf32 split (lo optional: tf32 alone), 2 = BF16 split
template <int OUT, bool FULL>
__device__ __forceinline__ void conv_store(const uint32_t (&r)[32], float* out_hi, float* out_lo, int64_t o0,
                                           int64_t step, int nj) {
    if constexpr (OUT == 2) {
        __nv_bfloat16* ph = reinterpret_cast<__nv_bfloat16*>(out_hi) + o0;
        __nv_bfloat16* pl = reinterpret_cast<__nv_bfloat16*>(out_lo) + o0;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            if (FULL || j < nj) {
                const float v = __uint_as_float(r[j]);
                const __nv_bfloat16 h = __float2bfloat16_rn(v);
                *ph = h;
                *pl = __float2bfloat16_rn(v - __bfloat162float(h));
            }
            ph += step;
            pl += step;
        }
    } else if constexpr (OUT == 1) {
        float* ph = out_hi + o0;
        float* pl = out_lo ? out_lo + o0 : nullptr;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            if (FULL || j < nj) {
                const float v = __uint_as_float(r[j]);
                uint32_t h;
                asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
                ph[(int64_t)j * step] = __uint_as_float(h);
                if (pl) pl[(int64_t)j * step] = v - __uint_as_float(h);
            }
        }
    } else {
        float* ph = out_hi + o0;
#pragma unroll
        for (int j = 0; j < 32; ++j)
            if (FULL || j < nj) ph[(int64_t)j * step] = __uint_as_float(r[j]);
    }
}

template <bool ALO, bool BF16, int OUT>
__global__ void __launch_bounds__(kConvThreads, 1)
umma_basis_conv(const __grid_constant__ CUtensorMap tA_hi, const __grid_constant__ CUtensorMap tA_lo,
                const __grid_constant__ CUtensorMap tS_hi, const __grid_constant__ CUtensorMap tS_lo, ConvArgs args) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[kConvStages], empty_bar[kConvStages], tfull_bar[2], tempty_bar[2];
    __shared__ __align__(8) uint64_t band_bar, drain_bar;
    __shared__ uint32_t tmem_base_s;
    __shared__ int abort_raw;
    volatile int& abort_s = abort_raw;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int TW = args.tw, KC = args.kc, KS = args.ks, KG = args.kg, NCG = args.ncg;
    const int NB = KG * TW;                               // band rows per K-step (N of a full group)
    const uint32_t bbytes = (uint32_t)NB * 64u;           // one K-step's band tile (a multiple of 1024)
    const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
    const uint32_t b_hi = base, b_lo = base + (uint32_t)KS * bbytes;
    const uint32_t stage0 = base + 2u * (uint32_t)KS * bbytes;
    auto sA_hi = [&](int s) { return stage0 + (uint32_t)s * 2u * kTileA; };
    auto sA_lo = [&](int s) { return stage0 + (uint32_t)s * 2u * kTileA + kTileA; };
    // this CTA's component group and its walk over the (rows, times) blocks
    const int cg = blockIdx.x % NCG, cta_step = gridDim.x / NCG;
    const int nblocks = ((args.nrows + kBM - 1) / kBM) * args.ntiles_w;
    const int blk0 = (int)(blockIdx.x / NCG);
    const int ng = min(KG, KC - cg * KG);                 // components of this group
    int* err = args.err;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kConvStages; ++s) {
            mbar_init(smem_u32(&full_bar[s]), 1);
            mbar_init(smem_u32(&empty_bar[s]), 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(smem_u32(&tfull_bar[a]), 1);
            mbar_init(smem_u32(&tempty_bar[a]), kConvEpiWarps);   // one arrival per epilogue warp
        }
        mbar_init(smem_u32(&band_bar), 1);
        mbar_init(smem_u32(&drain_bar), 1);
        abort_s = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_s;

    if (warp == kConvEpiWarps && lane == 0) {
        // ---- producer: the group's band tiles once, then the A tiles of every block of this CTA ----
        const uint32_t bb = smem_u32(&band_bar);
        mbar_expect_tx(bb, 2u * (uint32_t)KS * bbytes);
        for (int s = 0; s < KS; ++s) {
            tma_load_2d(b_hi + (uint32_t)s * bbytes, &tS_hi, bb, 0, (cg * KS + s) * NB);
            tma_load_2d(b_lo + (uint32_t)s * bbytes, &tS_lo, bb, 0, (cg * KS + s) * NB);
        }
        int q = 0;
        for (int blk = blk0; blk < nblocks && !abort_s; blk += cta_step) {
            const int mt = blk / args.ntiles_w, wt = blk - mt * args.ntiles_w;
            const int m0 = mt * kBM, x0 = wt * TW - args.hr;   // 16-byte aligned (hr and TW are)
            constexpr int kStep = BF16 ? 2 * kBK : kBK;         // input times per K-step
            bool stop = false;
            for (int ks = 0; ks < KS; ++ks, ++q) {
                const int s = q % kConvStages;
                const uint32_t round = (uint32_t)(q / kConvStages);
                if (!mbar_wait(smem_u32(&empty_bar[s]), (round & 1u) ^ 1u) || abort_s) {
                    atomicOr(err, 1);
                    abort_s = 1;
                    stop = true;
                    break;
                }
                const uint32_t fb = smem_u32(&full_bar[s]);
                mbar_expect_tx(fb, ALO ? 2u * kTileA : (uint32_t)kTileA);
                tma_load_2d(sA_hi(s), &tA_hi, fb, x0 + kStep * ks, m0);
                if constexpr (ALO) tma_load_2d(sA_lo(s), &tA_lo, fb, x0 + kStep * ks, m0);
            }
            if (stop) break;
        }
        // the copies of the last rounds and the bands land before the CTA may exit
        for (int kt = (q > kConvStages ? q - kConvStages : 0); kt < q; ++kt)
            if (!mbar_wait(smem_u32(&full_bar[kt % kConvStages]), (uint32_t)(kt / kConvStages) & 1u)) atomicOr(err, 4);
        if (!mbar_wait(bb, 0u)) atomicOr(err, 4);
    } else if (warp == kConvEpiWarps + 1 && lane == 0) {
        // ---- MMA issuer: per K-step one MMA of N = ng TW per product ----
        const uint32_t idesc = idesc_n(BF16 ? ((1u << 4) | (1u << 7) | (1u << 10)) : ((1u << 4) | (2u << 7) | (2u << 10)),
                                       ng * TW);
        if (!mbar_wait(smem_u32(&band_bar), 0u)) {
            atomicOr(err, 2);
            abort_s = 1;
        }
        int q = 0, i = 0;
        for (int blk = blk0; blk < nblocks && !abort_s; blk += cta_step, ++i) {
            const int ab = i & 1;
            if (!mbar_wait(smem_u32(&tempty_bar[ab]), ((uint32_t)(i >> 1) & 1u) ^ 1u) || abort_s) {
                atomicOr(err, 2);
                abort_s = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t d = tmem + (uint32_t)(ab * NB);
            bool stop = false;
            for (int ks = 0; ks < KS; ++ks, ++q) {
                const int s = q % kConvStages;
                const uint32_t round = (uint32_t)(q / kConvStages);
                if (!mbar_wait(smem_u32(&full_bar[s]), round & 1u) || abort_s) {
                    atomicOr(err, 2);
                    abort_s = 1;
                    stop = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
                for (int kk = 0; kk < 2; ++kk) {          // 32 bytes (8 tf32 / 16 bf16) per MMA
                    const uint32_t off = (uint32_t)kk * 32u;
                    const uint64_t ah = smem_desc(sA_hi(s) + off), al = smem_desc(sA_lo(s) + off);
                    const uint64_t bh = smem_desc(b_hi + (uint32_t)ks * bbytes + off);
                    const uint64_t bl = smem_desc(b_lo + (uint32_t)ks * bbytes + off);
                    const uint32_t acc = (ks > 0 || kk > 0) ? 1u : 0u;
                    if constexpr (BF16) {
                        mma_bf16_rt(d, ah, bh, idesc, acc);
                        mma_bf16_rt(d, ah, bl, idesc, 1u);
                        if constexpr (ALO) mma_bf16_rt(d, al, bh, idesc, 1u);
                    } else {
                        mma_tf32_rt(d, ah, bh, idesc, acc);
                        mma_tf32_rt(d, ah, bl, idesc, 1u);
                        if constexpr (ALO) mma_tf32_rt(d, al, bh, idesc, 1u);
                    }
                }
                mma_commit(smem_u32(&empty_bar[s]));
            }
            if (stop) break;
            mma_commit(smem_u32(&tfull_bar[ab]));
        }
        // every MMA issued has finished before the TMEM is released
        mma_commit(smem_u32(&drain_bar));
        if (!mbar_wait(smem_u32(&drain_bar), 0u)) atomicOr(err, 2);
    } else if (warp < kConvEpiWarps) {
        // ---- epilogue: accumulator -> Bpc ----
        const int quad = warp & 3;
        const int cpc = TW / 32;                          // 32-column chunks per component
        int i = 0;
        for (int blk = blk0; blk < nblocks; blk += cta_step, ++i) {
            const int ab = i & 1;
            // one decision per warp: the tcgen05.ld below is .sync.aligned
            const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&tfull_bar[ab]), (uint32_t)(i >> 1) & 1u) && !abort_s);
            if (!ok) {
                if (lane == 0) atomicOr(err, 8);
                abort_s = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int mt = blk / args.ntiles_w, wt = blk - mt * args.ntiles_w;
            const int row = mt * kBM + quad * 32 + lane, w0 = wt * TW;
            const int b = row / args.chans, ch = row - b * args.chans;
            for (int cc = warp >> 2; cc < ng * cpc; cc += kConvEpiWarps / 4) {
                // 32 output times of one component per chunk: (g, part) = (cc / cpc, cc % cpc)
                const int g = cc / cpc, c = cg * KG + g, wh = w0 + 32 * (cc - g * cpc);
                const int nj = min(32, args.wlen - wh);
                uint32_t r[32];
                const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(ab * NB + cc * 32);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                    "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
                    "[%32];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                      "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                      "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                      "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                    : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (row < args.nrows) {
                    // lanes = consecutive channels of one (w, k): 64- or 128-byte stores
                    const int64_t o0 = (((int64_t)b * args.wlen + wh) * KC + c) * args.chans + ch;
                    const int64_t step = (int64_t)KC * args.chans;
                    if (nj == 32)
                        conv_store<OUT, true>(r, args.out_hi, args.out_lo, o0, step, 32);
                    else
                        conv_store<OUT, false>(r, args.out_hi, args.out_lo, o0, step, nj);
                }
            }
            // the accumulator may be overwritten once every epilogue warp has read it
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&tempty_bar[ab]));
        }
    }
    __syncwarp();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
}

// hi = bf16(x) (round to nearest even), lo = bf16(x - hi)
__global__ void split_bf16_kernel(const float* __restrict__ x, __nv_bfloat16* __restrict__ hi,
                                  __nv_bfloat16* __restrict__ lo, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = x[i];
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        hi[i] = h;
        lo[i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

void launch_split_bf16(const float* x, void* hi, void* lo, int64_t n, cudaStream_t s) {
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
    split_bf16_kernel<<<blocks, 256, 0, s>>>(x, static_cast<__nv_bfloat16*>(hi), static_cast<__nv_bfloat16*>(lo), n);
}

void launch_split_tf32(const float* x, float* hi, float* lo, int64_t n, cudaStream_t s) {
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
    split_tf32_kernel<<<blocks, 256, 0, s>>>(x, hi, lo, n);
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// rows x cols fp32 row-major, boxes of 16 columns (64 B) x box_rows rows, 64-byte swizzle
bool make_map(CUtensorMap* m, const float* ptr, uint64_t rows, uint64_t cols, uint32_t box_rows) {
    auto fn = encode_fn();
    if (!fn || ((uintptr_t)ptr & 15) || (cols * 4) % 16) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 4};
    const cuuint32_t box[2] = {(cuuint32_t)kBK, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)ptr, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

// rows x cols bf16 row-major, boxes of 32 columns (64 B) x box_rows rows, 64-byte swizzle
static bool make_map_bf16(CUtensorMap* m, const void* ptr, uint64_t rows, uint64_t cols, uint32_t box_rows) {
    auto fn = encode_fn();
    if (!fn || ((uintptr_t)ptr & 15) || (cols * 2) % 16) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 2};
    const cuuint32_t box[2] = {(cuuint32_t)(2 * kBK), box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)ptr, dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// rows x cols bytes (FP8) row-major, boxes of 64 columns (64 B) x box_rows rows, 64-byte swizzle
static bool make_map_u8(CUtensorMap* m, const void* ptr, uint64_t rows, uint64_t cols, uint32_t box_rows) {
    auto fn = encode_fn();
    if (!fn || ((uintptr_t)ptr & 15) || cols % 16) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols};
    const cuuint32_t box[2] = {(cuuint32_t)(4 * kBK), box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, (void*)ptr, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

struct UmmaOperands {
    CUtensorMap a_hi, a_lo, b_hi, b_lo;
    bool bf16 = false;        // BF16 splits (kind::f16) instead of TF32 splits
    bool has_a_lo = true;     // false: A is TF32 data alone (two products)
    int lowp = 0;             // 1 = one BF16 product of the hi parts, 2 = one FP8 e4m3 product
    const float* col_scale = nullptr;   // per output column (B row) scale applied in the epilogue
    int rows_a = 0, rows_b = 0, K = 0;
    int cols_a = 0;           // Toeplitz: columns of A (wrapped window length, padded)
    int bn = 256;             // plain mode: output columns per tile (the B map's box rows)
};

constexpr int kPlainBN = 256;
constexpr int kNarrowBN = 192;
// output columns per tile of a plain GEMM with N columns: 192 where it tiles N exactly (192, 384:
// the whitening of 384 channels wastes no quarter of its MMAs on padding), else 256
static int plain_bn(int64_t n) { return (n == kNarrowBN || n == 2 * kNarrowBN) ? kNarrowBN : kPlainBN; }
template <int BN>
constexpr int smem_bytes() {
    return (kSmemBudget / (2 * kTileA + 2 * BN * kBK * 4)) * (2 * kTileA + 2 * BN * kBK * 4) + 1024;
}
template <int BN>
constexpr int smem_bytes_lowp() {
    return (kSmemBudget / (kTileA + BN * kBK * 4)) * (kTileA + BN * kBK * 4) + 1024;
}

UmmaOperands* umma_make(const float* a_hi, const float* a_lo, int64_t rows_a, const float* b_hi, const float* b_lo,
                        int64_t rows_b, int K) {
    if (K % kBK != 0 || rows_b > 2 * kPlainBN) return nullptr;
    auto* u = new UmmaOperands();
    u->rows_a = (int)rows_a;
    u->rows_b = (int)rows_b;
    u->K = K;
    u->bn = plain_bn(rows_b);
    u->has_a_lo = a_lo != nullptr;
    if (!a_lo) a_lo = a_hi;   // the map is never used
    if (!make_map(&u->a_hi, a_hi, rows_a, K, kBM) || !make_map(&u->a_lo, a_lo, rows_a, K, kBM) ||
        !make_map(&u->b_hi, b_hi, rows_b, K, u->bn) || !make_map(&u->b_lo, b_lo, rows_b, K, u->bn)) {
        delete u;
        return nullptr;
    }
    return u;
}

UmmaOperands* umma_make_bf16(const void* a_hi, const void* a_lo, int64_t rows_a, const void* b_hi, const void* b_lo,
                             int64_t rows_b, int K) {
    if (K % (2 * kBK) != 0 || rows_b > 2 * kPlainBN || !a_lo || !b_lo) return nullptr;
    auto* u = new UmmaOperands();
    u->bf16 = true;
    u->rows_a = (int)rows_a;
    u->rows_b = (int)rows_b;
    u->K = K;
    u->bn = plain_bn(rows_b);
    if (!make_map_bf16(&u->a_hi, a_hi, rows_a, K, kBM) || !make_map_bf16(&u->a_lo, a_lo, rows_a, K, kBM) ||
        !make_map_bf16(&u->b_hi, b_hi, rows_b, K, u->bn) || !make_map_bf16(&u->b_lo, b_lo, rows_b, K, u->bn)) {
        delete u;
        return nullptr;
    }
    return u;
}

UmmaOperands* umma_make_lowp(const void* a, int64_t rows_a, const void* b, int64_t rows_b, int K, int lowp,
                             const float* col_scale) {
    const int ke = lowp == 2 ? 4 * kBK : 2 * kBK;   // elements per 64-byte K-step
    if ((lowp != 1 && lowp != 2) || K % ke != 0 || rows_b > 2 * kPlainBN) return nullptr;
    auto* u = new UmmaOperands();
    u->bf16 = lowp == 1;
    u->lowp = lowp;
    u->rows_a = (int)rows_a;
    u->rows_b = (int)rows_b;
    u->K = K;
    const bool ok = lowp == 2 ? make_map_u8(&u->a_hi, a, rows_a, K, kBM) && make_map_u8(&u->b_hi, b, rows_b, K, kPlainBN)
                              : make_map_bf16(&u->a_hi, a, rows_a, K, kBM) && make_map_bf16(&u->b_hi, b, rows_b, K, kPlainBN);
    if (!ok) {
        delete u;
        return nullptr;
    }
    u->a_lo = u->a_hi;   // never loaded
    u->b_lo = u->b_hi;
    u->col_scale = col_scale;
    return u;
}

UmmaOperands* umma_make_toeplitz_bf16(const void* x_hi, const void* x_lo, int64_t rows, int64_t cols, int tile,
                                      const void* g_hi, const void* g_lo, int K) {
    if (K % (2 * kBK) != 0 || cols % 8 != 0 || !x_lo || !g_lo ||
        (tile != kHighpassTileSmall && tile != kHighpassTileLarge))
        return nullptr;
    auto* u = new UmmaOperands();
    u->bf16 = true;
    u->rows_a = (int)rows;
    u->cols_a = (int)cols;
    u->rows_b = tile;
    u->K = K;
    if (!make_map_bf16(&u->a_hi, x_hi, rows, cols, kBM) || !make_map_bf16(&u->a_lo, x_lo, rows, cols, kBM) ||
        !make_map_bf16(&u->b_hi, g_hi, tile, K, tile) || !make_map_bf16(&u->b_lo, g_lo, tile, K, tile)) {
        delete u;
        return nullptr;
    }
    return u;
}

UmmaOperands* umma_make_toeplitz(const float* x_hi, const float* x_lo, int64_t rows, int64_t cols, int tile,
                                 const float* g_hi, const float* g_lo, int K) {
    if (K % kBK != 0 || cols % 4 != 0 || (tile != kHighpassTileSmall && tile != kHighpassTileLarge)) return nullptr;
    auto* u = new UmmaOperands();
    u->rows_a = (int)rows;
    u->cols_a = (int)cols;
    u->rows_b = tile;
    u->K = K;
    u->has_a_lo = x_lo != nullptr;
    if (!x_lo) x_lo = x_hi;   // the map is never used
    if (!make_map(&u->a_hi, x_hi, rows, cols, kBM) || !make_map(&u->a_lo, x_lo, rows, cols, kBM) ||
        !make_map(&u->b_hi, g_hi, tile, K, tile) || !make_map(&u->b_lo, g_lo, tile, K, tile)) {
        delete u;
        return nullptr;
    }
    return u;
}

void umma_free(UmmaOperands* u) { delete u; }

// persistent GEMM grid: one CTA per SM (each holds 2 x BN TMEM columns and most of the shared
// memory), fewer when there are fewer tiles
static cudaError_t gemm_grid(int64_t ntiles, int& grid) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, std::max(sms, 1)));
    return cudaSuccess;
}

cudaError_t launch_umma_gemm(const UmmaOperands* u, float* Cm, int M, int N, int64_t ldc, int* err, cudaStream_t s) {
    return launch_umma_gemm_zt(u, Cm, M, N, ldc, nullptr, nullptr, 1, 0, err, s);
}

template <int BN>
static cudaError_t launch_zt_bn(const UmmaOperands* u, float* Cm, int M, int N, int64_t ldc, float* zt_hi,
                                float* zt_lo, int wlen, int zpitch, int* err, cudaStream_t s, bool zt_bf16) {
    void (*kern)(CUtensorMap, CUtensorMap, CUtensorMap, CUtensorMap, UmmaArgs) = nullptr;
    if constexpr (BN == kPlainBN) {
        kern = u->lowp == 2  ? umma_gemm_3xtf32<BN, kPlain, true, false, 2>
               : u->lowp == 1 ? umma_gemm_3xtf32<BN, kPlain, true, true, 1>
               : u->bf16     ? umma_gemm_3xtf32<BN, kPlain, true, true>
               : u->has_a_lo ? umma_gemm_3xtf32<BN, kPlain, true>
                             : umma_gemm_3xtf32<BN, kPlain, false>;
    } else {
        if (u->lowp) return cudaErrorInvalidValue;   // the low-precision operands are made with 256-row tiles
        kern = u->bf16 ? umma_gemm_3xtf32<BN, kPlain, true, true>
               : u->has_a_lo ? umma_gemm_3xtf32<BN, kPlain, true>
                             : umma_gemm_3xtf32<BN, kPlain, false>;
    }
    const int smem = u->lowp ? smem_bytes_lowp<BN>() : smem_bytes<BN>();
    const cudaError_t attr_err = raise_smem_limit((const void*)kern, smem);
    if (attr_err != cudaSuccess) return attr_err;
    UmmaArgs a{};
    a.out = Cm;
    a.M = M;
    a.N = N;
    a.K = u->K;
    a.ldc = ldc;
    a.err = err;
    a.zt_hi = zt_hi;
    a.zt_lo = zt_lo;
    a.wlen = wlen;
    a.zpitch = zpitch;
    a.zt_bf16 = zt_bf16 ? 1 : 0;
    a.col_scale = u->col_scale;
    a.slices = 1;
    int grid = 0;
    const cudaError_t ge = gemm_grid((int64_t)((N + BN - 1) / BN) * ((M + kBM - 1) / kBM), grid);
    if (ge != cudaSuccess) return ge;
    kern<<<grid, kGemmThreads, smem, s>>>(u->a_hi, u->a_lo, u->b_hi, u->b_lo, a);
    return cudaGetLastError();
}

cudaError_t launch_umma_gemm_zt(const UmmaOperands* u, float* Cm, int M, int N, int64_t ldc, float* zt_hi,
                                float* zt_lo, int wlen, int zpitch, int* err, cudaStream_t s, bool zt_bf16) {
    if (!u || M > u->rows_a || N > u->rows_b || N > 2 * kPlainBN) return cudaErrorInvalidValue;
    if (zt_hi && (wlen <= 0 || zpitch < wlen || (zt_bf16 && !zt_lo))) return cudaErrorInvalidValue;
    if (!Cm && !zt_hi) return cudaErrorInvalidValue;
    if (u->bn == kNarrowBN)
        return launch_zt_bn<kNarrowBN>(u, Cm, M, N, ldc, zt_hi, zt_lo, wlen, zpitch, err, s, zt_bf16);
    return launch_zt_bn<kPlainBN>(u, Cm, M, N, ldc, zt_hi, zt_lo, wlen, zpitch, err, s, zt_bf16);
}

// C[m][n] = sum over the slices of ws[s][m][n], in slice order
__global__ void sum_slices_kernel(const float* __restrict__ ws, float* __restrict__ Cm, int M, int N, int64_t ldc,
                                  int S) {
    const int64_t total = (int64_t)M * N;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t m = i / N, n = i - m * N;
        float acc = ws[m * ldc + n];
        for (int s = 1; s < S; ++s) acc += ws[((int64_t)s * M + m) * ldc + n];
        Cm[m * ldc + n] = acc;
    }
}

template <int BN>
static cudaError_t launch_splitk_bn(const UmmaOperands* u, float* Cm, int M, int N, int64_t ldc, float* ws, int S,
                                   int* err, cudaStream_t s) {
    void (*kern)(CUtensorMap, CUtensorMap, CUtensorMap, CUtensorMap, UmmaArgs) = nullptr;
    if constexpr (BN == kPlainBN) {
        kern = u->lowp == 2  ? umma_gemm_3xtf32<BN, kPlain, true, false, 2>
               : u->lowp == 1 ? umma_gemm_3xtf32<BN, kPlain, true, true, 1>
               : u->bf16     ? umma_gemm_3xtf32<BN, kPlain, true, true>
               : u->has_a_lo ? umma_gemm_3xtf32<BN, kPlain, true>
                             : umma_gemm_3xtf32<BN, kPlain, false>;
    } else {
        if (u->lowp) return cudaErrorInvalidValue;
        kern = u->bf16 ? umma_gemm_3xtf32<BN, kPlain, true, true>
               : u->has_a_lo ? umma_gemm_3xtf32<BN, kPlain, true>
                             : umma_gemm_3xtf32<BN, kPlain, false>;
    }
    const int smem = u->lowp ? smem_bytes_lowp<BN>() : smem_bytes<BN>();
    const cudaError_t attr_err = raise_smem_limit((const void*)kern, smem);
    if (attr_err != cudaSuccess) return attr_err;
    UmmaArgs a{};
    a.out = ws;
    a.M = M;
    a.N = N;
    a.K = u->K;
    a.ldc = ldc;
    a.err = err;
    a.wlen = 1;
    a.col_scale = u->col_scale;   // the slices are scaled before they are summed: sum(s x) = s sum(x) up to rounding
    a.slices = S;
    int grid = 0;
    const cudaError_t ge = gemm_grid((int64_t)((N + BN - 1) / BN) * ((M + kBM - 1) / kBM) * S, grid);
    if (ge != cudaSuccess) return ge;
    kern<<<grid, kGemmThreads, smem, s>>>(u->a_hi, u->a_lo, u->b_hi, u->b_lo, a);
    const int blocks = (int)std::min<int64_t>(((int64_t)M * N + 255) / 256, 2048);
    sum_slices_kernel<<<blocks, 256, 0, s>>>(ws, Cm, M, N, ldc, S);
    return cudaGetLastError();
}

cudaError_t launch_umma_gemm_splitk(const UmmaOperands* u, float* Cm, int M, int N, int64_t ldc, float* ws, int S,
                                    int* err, cudaStream_t s) {
    if (!u || M > u->rows_a || N > u->rows_b || N > 2 * kPlainBN || S < 1 || !ws)
        return cudaErrorInvalidValue;
    const int nk = u->K / (u->lowp == 2 ? 4 * kBK : (u->bf16 ? 2 * kBK : kBK));
    S = std::min(S, nk);
    if (S <= 1) return launch_umma_gemm(u, Cm, M, N, ldc, err, s);
    if (u->bn == kNarrowBN) return launch_splitk_bn<kNarrowBN>(u, Cm, M, N, ldc, ws, S, err, s);
    return launch_splitk_bn<kPlainBN>(u, Cm, M, N, ldc, ws, S, err, s);
}

// Y[b][w][c] (tf32 split) = circular high-pass of nb windows held channel-major in the operands
template <int TILE>
static cudaError_t launch_highpass_tile(const UmmaOperands* u, float* Y_hi, float* Y_lo, int nb, int C, int W,
                                        int* err, cudaStream_t s) {
    auto kern = u->bf16       ? umma_gemm_3xtf32<TILE, kToeplitz, true, true>
                : u->has_a_lo ? umma_gemm_3xtf32<TILE, kToeplitz, true>
                              : umma_gemm_3xtf32<TILE, kToeplitz, false>;
    constexpr int smem = smem_bytes<TILE>();
    const cudaError_t attr_err = raise_smem_limit((const void*)kern, smem);
    if (attr_err != cudaSuccess) return attr_err;
    UmmaArgs a{};
    a.out = Y_hi;
    a.out_lo = Y_lo;
    a.M = nb * C;
    a.N = W;
    a.K = u->K;
    a.chans = C;
    a.wlen = W;
    a.err = err;
    a.slices = 1;
    int grid = 0;
    const cudaError_t ge = gemm_grid((int64_t)((W + TILE - 1) / TILE) * ((nb * C + kBM - 1) / kBM), grid);
    if (ge != cudaSuccess) return ge;
    kern<<<grid, kGemmThreads, smem, s>>>(u->a_hi, u->a_lo, u->b_hi, u->b_lo, a);
    return cudaGetLastError();
}

cudaError_t launch_umma_highpass(const UmmaOperands* u, float* Y_hi, float* Y_lo, int nb, int C, int W, int* err,
                                 cudaStream_t s) {
    if (!u || nb * C > u->rows_a) return cudaErrorInvalidValue;
    if (u->rows_b == kHighpassTileLarge)
        return launch_highpass_tile<kHighpassTileLarge>(u, Y_hi, Y_lo, nb, C, W, err, s);
    return launch_highpass_tile<kHighpassTileSmall>(u, Y_hi, Y_lo, nb, C, W, err, s);
}

// ---- tensor-core basis convolution: geometry, band tiles, maps, launch ----
bool conv_tc_geometry(int nt, int K, ConvGeometry& g, bool bf16) {
    if (K < 1 || K > kConvMaxK || nt < 1) return false;
    const int H = nt / 2;
    const int step = bf16 ? 2 * kBK : kBK;
    const int al = bf16 ? 8 : 4;                       // elements in 16 bytes
    const int hr = (H + al - 1) / al * al;             // tile inputs start 16-byte aligned
    // the tile width and component grouping with the fewest MMAs per output (K-steps per tile over
    // the kg TW outputs a K-step's MMA covers), within N <= 256 (two accumulators fit the 512 TMEM
    // columns) and the shared-memory budget; ties go to the wider tile
    bool found = false;
    double best = 0.0;
    for (int tw : {64, 32}) {
        const int ks = (tw + nt - 1 + (hr - H) + step - 1) / step;
        for (int ncg = 1; ncg <= K; ++ncg) {
            const int kg = (K + ncg - 1) / ncg;
            if (kg * tw > 256) continue;
            const size_t smem = 1024 + 2 * (size_t)ks * kg * tw * 64 + (size_t)kConvStages * 2 * kTileA;
            if (smem > (size_t)kConvSmemMax) continue;
            const double cost = (double)ks / (kg * tw);
            if (!found || cost < best) {
                found = true;
                best = cost;
                g.bf16 = bf16;
                g.step = step;
                g.tw = tw;
                g.ks = ks;
                g.hr = hr;
                g.kg = kg;
                g.ncg = ncg;
                g.rows = ncg * ks * kg * tw;
            }
            break;   // more groups only narrow the MMA
        }
    }
    return found;
}

void conv_tc_bands(const float* wPCA, int K, int nt, const ConvGeometry& g, float* bands) {
    const int d = g.hr - nt / 2;
    const int nb = g.kg * g.tw;
    for (int cg = 0; cg < g.ncg; ++cg)
        for (int s = 0; s < g.ks; ++s)
            for (int n = 0; n < nb; ++n) {
                const int k = cg * g.kg + n / g.tw, j = n % g.tw;
                float* row = bands + ((size_t)(cg * g.ks + s) * nb + n) * g.step;
                for (int i = 0; i < g.step; ++i) {
                    const int m = g.step * s + i - j - d;
                    row[i] = (k < K && m >= 0 && m < nt) ? wPCA[(size_t)k * nt + m] : 0.f;
                }
            }
}

struct ConvOperands {
    CUtensorMap a_hi, a_lo, s_hi, s_lo;
    bool has_a_lo = true;
    int K = 0;
    ConvGeometry g;
    int64_t rows = 0;
    int wlen = 0;
};

// rows x cols fp32 at a row pitch of `pitch` floats: TMA fills columns >= cols (and < 0) with zeros
static bool make_map_pitched(CUtensorMap* m, const float* ptr, uint64_t rows, uint64_t cols, uint64_t pitch,
                             uint32_t box_rows) {
    auto fn = encode_fn();
    if (!fn || ((uintptr_t)ptr & 15) || (pitch * 4) % 16 || pitch < cols) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {pitch * 4};
    const cuuint32_t box[2] = {(cuuint32_t)kBK, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)ptr, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

// the same for bf16 elements
static bool make_map_pitched_bf16(CUtensorMap* m, const void* ptr, uint64_t rows, uint64_t cols, uint64_t pitch,
                                  uint32_t box_rows) {
    auto fn = encode_fn();
    if (!fn || ((uintptr_t)ptr & 15) || (pitch * 2) % 16 || pitch < cols) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {pitch * 2};
    const cuuint32_t box[2] = {(cuuint32_t)(2 * kBK), box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)ptr, dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

ConvOperands* conv_tc_make(const float* zt_hi, const float* zt_lo, int64_t rows, int wlen, int zpitch,
                           const float* s_hi, const float* s_lo, int K, const ConvGeometry& g) {
    if (g.bf16) {
        // BF16 splits: A and the band tiles are bf16 arrays (the three products need both lo parts)
        if (!zt_lo) return nullptr;
        auto* u = new ConvOperands();
        u->K = K;
        u->g = g;
        u->rows = rows;
        u->wlen = wlen;
        if (!make_map_pitched_bf16(&u->a_hi, zt_hi, rows, wlen, zpitch, kBM) ||
            !make_map_pitched_bf16(&u->a_lo, zt_lo, rows, wlen, zpitch, kBM) ||
            !make_map_bf16(&u->s_hi, s_hi, (uint64_t)g.rows, g.step, g.kg * g.tw) ||
            !make_map_bf16(&u->s_lo, s_lo, (uint64_t)g.rows, g.step, g.kg * g.tw)) {
            delete u;
            return nullptr;
        }
        return u;
    }
    auto* u = new ConvOperands();
    u->has_a_lo = zt_lo != nullptr;
    u->K = K;
    u->g = g;
    u->rows = rows;
    u->wlen = wlen;
    if (!zt_lo) zt_lo = zt_hi;   // the map is never used
    if (!make_map_pitched(&u->a_hi, zt_hi, rows, wlen, zpitch, kBM) ||
        !make_map_pitched(&u->a_lo, zt_lo, rows, wlen, zpitch, kBM) ||
        !make_map(&u->s_hi, s_hi, (uint64_t)g.rows, 16, g.kg * g.tw) ||
        !make_map(&u->s_lo, s_lo, (uint64_t)g.rows, 16, g.kg * g.tw)) {
        delete u;
        return nullptr;
    }
    return u;
}

void conv_tc_free(ConvOperands* u) { delete u; }

cudaError_t launch_umma_basis_conv(const ConvOperands* u, float* out_hi, float* out_lo, bool hi_only, int nb, int C,
                                   int W, int* err, cudaStream_t s, bool out_bf16) {
    if (!u || (int64_t)nb * C > u->rows || W != u->wlen || nb <= 0 || (out_bf16 && !out_lo))
        return cudaErrorInvalidValue;
    // the BF16 operands always come with the BF16 split output (the BF16 projection reads it)
    if (u->g.bf16 != out_bf16) return cudaErrorInvalidValue;
    auto kern = u->g.bf16 ? umma_basis_conv<true, true, 2>
                : (out_lo || hi_only) ? (u->has_a_lo ? umma_basis_conv<true, false, 1> : umma_basis_conv<false, false, 1>)
                                      : (u->has_a_lo ? umma_basis_conv<true, false, 0> : umma_basis_conv<false, false, 0>);
    // at least 120 KB, so that one CTA (holding all 512 TMEM columns) runs per SM
    const ConvGeometry& g = u->g;
    const int smem = std::max<int>(120 * 1024, 1024 + 2 * g.ks * g.kg * g.tw * 64 + kConvStages * 2 * kTileA);
    const cudaError_t attr_err = raise_smem_limit((const void*)kern, smem);
    if (attr_err != cudaSuccess) return attr_err;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    ConvArgs a{};
    a.out_hi = out_hi;
    a.out_lo = out_lo;
    a.nrows = nb * C;
    a.chans = C;
    a.wlen = W;
    a.kc = u->K;
    a.ks = g.ks;
    a.hr = g.hr;
    a.tw = g.tw;
    a.kg = g.kg;
    a.ncg = g.ncg;
    a.ntiles_w = (W + g.tw - 1) / g.tw;
    a.err = err;
    // a multiple of ncg CTAs: CTA b serves group b % ncg over every ncg-th block
    const int64_t nblocks = (int64_t)((nb * C + kBM - 1) / kBM) * a.ntiles_w;
    const int64_t per_group = std::max<int64_t>(1, std::min<int64_t>(nblocks, std::max(sms, g.ncg) / g.ncg));
    const int grid = (int)(per_group * g.ncg);
    kern<<<grid, kConvThreads, smem, s>>>(u->a_hi, u->a_lo, u->s_hi, u->s_lo, a);
    return cudaGetLastError();
}

}  // namespace lss
