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
// One CTA (4 warps) computes a 128 x N tile: warp 0 / lane 0 streams A and B tiles into shared
// memory with TMA (cp.async.bulk.tensor, 64-byte swizzle) through a 4-stage mbarrier pipeline;
// warp 1 / lane 0 issues tcgen05.mma.kind::tf32 (M = 128, N = 128 or 256, K = 8) into an N-column
// TMEM accumulator and releases each stage with tcgen05.commit; all four warps then read the
// accumulator back with tcgen05.ld (each warp its 32 TMEM lanes = tile rows) and store it.
// Every wait is bounded (globaltimer); on a timeout the kernel sets an error word, waits (bounded)
// for the copies it issued, frees its TMEM and returns.
#include "lss_kernels.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

namespace lss {

constexpr int kBM = 128, kBK = 16;
constexpr int kTileA = kBM * kBK * 4;                   // 8 KB
constexpr int kSmemBudget = 196 * 1024;                 // stage buffers per CTA
constexpr uint64_t kWaitNs = 2000000000ull;             // 2 s

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
// fixed B operand keeps its split), for the tensor-core tier whose activations are stored once
template <int BN, int MODE, bool ALO>
__global__ void __launch_bounds__(128, 1)
umma_gemm_3xtf32(const __grid_constant__ CUtensorMap tA_hi, const __grid_constant__ CUtensorMap tA_lo,
                 const __grid_constant__ CUtensorMap tB_hi, const __grid_constant__ CUtensorMap tB_lo, UmmaArgs args) {
    constexpr int kBN = BN;
    constexpr int kTileB = kBN * kBK * 4;
    constexpr int kStageBytes = 2 * kTileA + 2 * kTileB;
    constexpr int kLoadBytes = ALO ? kStageBytes : kTileA + 2 * kTileB;   // bytes the TMA lands per stage
    constexpr int kStages = kSmemBudget / kStageBytes;
    const int M = args.M, N = args.N, K = args.K;
    int* err = args.err;
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages], done_bar;
    __shared__ uint32_t tmem_base_s;
    __shared__ int abort_raw;
    volatile int& abort_s = abort_raw;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.x * kBN, m0 = blockIdx.y * kBM;
    const int nk = K / kBK;
    // 1024-byte aligned stage buffers: [A_hi][A_lo][B_hi][B_lo] per stage
    const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
    auto sA_hi = [&](int s) { return base + (uint32_t)(s * kStageBytes); };
    auto sA_lo = [&](int s) { return base + (uint32_t)(s * kStageBytes + kTileA); };
    auto sB_hi = [&](int s) { return base + (uint32_t)(s * kStageBytes + 2 * kTileA); };
    auto sB_lo = [&](int s) { return base + (uint32_t)(s * kStageBytes + 2 * kTileA + kTileB); };

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(smem_u32(&full_bar[s]), 1);
            mbar_init(smem_u32(&empty_bar[s]), 1);
        }
        mbar_init(smem_u32(&done_bar), 1);
        abort_s = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                     "r"(kBN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_s;

    if (warp == 0 && lane == 0) {
        // ---- producer: TMA ----
        int issued = 0;
        for (int kt = 0; kt < nk; ++kt) {
            const int s = kt % kStages;
            const uint32_t round = (uint32_t)(kt / kStages);
            if (!mbar_wait(smem_u32(&empty_bar[s]), (round & 1u) ^ 1u) || abort_s) {
                atomicOr(err, 1);
                abort_s = 1;
                break;
            }
            const uint32_t fb = smem_u32(&full_bar[s]);
            mbar_expect_tx(fb, kLoadBytes);
            const int k0 = kt * kBK;   // a multiple of 16 fp32 = 64 bytes
            // Toeplitz: A columns start at the tile's output time n0 (a multiple of 128), B is the
            // same band matrix for every tile
            const int ax = (MODE == kToeplitz) ? n0 + k0 : k0;
            const int by = (MODE == kToeplitz) ? 0 : n0;
            tma_load_2d(sA_hi(s), &tA_hi, fb, ax, m0);
            if constexpr (ALO) tma_load_2d(sA_lo(s), &tA_lo, fb, ax, m0);
            tma_load_2d(sB_hi(s), &tB_hi, fb, k0, by);
            tma_load_2d(sB_lo(s), &tB_lo, fb, k0, by);
            ++issued;
        }
        // the copies of the last rounds must have landed before the CTA may exit
        for (int kt = (issued > kStages ? issued - kStages : 0); kt < issued; ++kt)
            if (!mbar_wait(smem_u32(&full_bar[kt % kStages]), (uint32_t)(kt / kStages) & 1u)) atomicOr(err, 4);
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        for (int kt = 0; kt < nk; ++kt) {
            const int s = kt % kStages;
            const uint32_t round = (uint32_t)(kt / kStages);
            if (!mbar_wait(smem_u32(&full_bar[s]), round & 1u) || abort_s) {
                atomicOr(err, 2);
                abort_s = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int kk = 0; kk < kBK / 8; ++kk) {          // K = 8 tf32 (32 bytes) per MMA
                const uint32_t off = (uint32_t)kk * 32u;
                const uint64_t ah = smem_desc(sA_hi(s) + off), al = smem_desc(sA_lo(s) + off);
                const uint64_t bh = smem_desc(sB_hi(s) + off), bl = smem_desc(sB_lo(s) + off);
                mma_tf32<BN>(tmem, ah, bh, (kt > 0 || kk > 0) ? 1u : 0u);
                mma_tf32<BN>(tmem, ah, bl, 1u);
                if constexpr (ALO) mma_tf32<BN>(tmem, al, bh, 1u);
            }
            mma_commit(smem_u32(&empty_bar[s]));        // frees the stage once these MMAs finish
        }
        mma_commit(smem_u32(&done_bar));
    }
    __syncwarp();

    // ---- epilogue: TMEM -> registers -> global ----
    const bool ok = mbar_wait(smem_u32(&done_bar), 0u) && !abort_s;
    if (!ok && threadIdx.x == 0) atomicOr(err, 8);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < kBN; c0 += 32) {
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
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
            if (ok && row < M) {
                const int b = row / args.chans, c = row - b * args.chans;
                for (int j = 0; j < 32; ++j) {
                    const int w = n0 + c0 + j;
                    if (w < args.wlen) {
                        const float v = __uint_as_float(r[j]);
                        uint32_t h;
                        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
                        const int64_t o = ((int64_t)b * args.wlen + w) * args.chans + c;
                        args.out[o] = __uint_as_float(h);
                        if (args.out_lo) args.out_lo[o] = v - __uint_as_float(h);
                    }
                }
            }
            continue;
        }
        if (ok && row < M) {
            float* crow = args.out + (int64_t)row * args.ldc + n0 + c0;
            const int ncol = min(32, N - (n0 + c0));
            if (ncol == 32 && ((((uintptr_t)crow) & 15) == 0)) {
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
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kBN) : "memory");
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

struct UmmaOperands {
    CUtensorMap a_hi, a_lo, b_hi, b_lo;
    bool has_a_lo = true;     // false: A is TF32 data alone (two products)
    int rows_a = 0, rows_b = 0, K = 0;
    int cols_a = 0;           // Toeplitz: columns of A (wrapped window length, padded)
};

constexpr int kPlainBN = 256;
template <int BN>
constexpr int smem_bytes() {
    return (kSmemBudget / (2 * kTileA + 2 * BN * kBK * 4)) * (2 * kTileA + 2 * BN * kBK * 4) + 1024;
}

UmmaOperands* umma_make(const float* a_hi, const float* a_lo, int64_t rows_a, const float* b_hi, const float* b_lo,
                        int64_t rows_b, int K) {
    if (K % kBK != 0 || rows_b > 2 * kPlainBN) return nullptr;
    auto* u = new UmmaOperands();
    u->rows_a = (int)rows_a;
    u->rows_b = (int)rows_b;
    u->K = K;
    u->has_a_lo = a_lo != nullptr;
    if (!a_lo) a_lo = a_hi;   // the map is never used
    if (!make_map(&u->a_hi, a_hi, rows_a, K, kBM) || !make_map(&u->a_lo, a_lo, rows_a, K, kBM) ||
        !make_map(&u->b_hi, b_hi, rows_b, K, kPlainBN) || !make_map(&u->b_lo, b_lo, rows_b, K, kPlainBN)) {
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

cudaError_t launch_umma_gemm(const UmmaOperands* u, float* Cm, int M, int N, int64_t ldc, int* err, cudaStream_t s) {
    if (!u || M > u->rows_a || N > u->rows_b || N > 2 * kPlainBN) return cudaErrorInvalidValue;
    auto kern = u->has_a_lo ? umma_gemm_3xtf32<kPlainBN, kPlain, true> : umma_gemm_3xtf32<kPlainBN, kPlain, false>;
    constexpr int smem = smem_bytes<kPlainBN>();
    const cudaError_t attr_err = raise_smem_limit((const void*)kern, smem);
    if (attr_err != cudaSuccess) return attr_err;
    UmmaArgs a{};
    a.out = Cm;
    a.M = M;
    a.N = N;
    a.K = u->K;
    a.ldc = ldc;
    a.err = err;
    dim3 grid((N + kPlainBN - 1) / kPlainBN, (M + kBM - 1) / kBM);
    kern<<<grid, 128, smem, s>>>(u->a_hi, u->a_lo, u->b_hi, u->b_lo, a);
    return cudaGetLastError();
}

// Y[b][w][c] (tf32 split) = circular high-pass of nb windows held channel-major in the operands
template <int TILE>
static cudaError_t launch_highpass_tile(const UmmaOperands* u, float* Y_hi, float* Y_lo, int nb, int C, int W,
                                        int* err, cudaStream_t s) {
    auto kern = u->has_a_lo ? umma_gemm_3xtf32<TILE, kToeplitz, true> : umma_gemm_3xtf32<TILE, kToeplitz, false>;
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
    dim3 grid((W + TILE - 1) / TILE, (nb * C + kBM - 1) / kBM);
    kern<<<grid, 128, smem, s>>>(u->a_hi, u->a_lo, u->b_hi, u->b_lo, a);
    return cudaGetLastError();
}

cudaError_t launch_umma_highpass(const UmmaOperands* u, float* Y_hi, float* Y_lo, int nb, int C, int W, int* err,
                                 cudaStream_t s) {
    if (!u || nb * C > u->rows_a) return cudaErrorInvalidValue;
    if (u->rows_b == kHighpassTileLarge)
        return launch_highpass_tile<kHighpassTileLarge>(u, Y_hi, Y_lo, nb, C, W, err, s);
    return launch_highpass_tile<kHighpassTileSmall>(u, Y_hi, Y_lo, nb, C, W, err, s);
}

}  // namespace lss
