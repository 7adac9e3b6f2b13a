// kernels_pre.cu -- preprocessing of a group of windows (Kilosort io.py:757-790):
// exact integer channel sums, mean removal + median CAR (one warp per time sample), the
// circular zero-phase high-pass as an FIR in registers, and the temporal-basis convolution
// (Kilosort template_matching.py:145, conv1d with padding nt//2).
#include "lss_kernels.cuh"
#include "lss_select.cuh"

#include <cuda_bf16.h>

#include <cstdio>

namespace lss {

// ---------------------------------------------------------------------------------------
// channel means over each window: exact integer sums, then mean = q + r / W in FP32 (q, r the
// integer quotient and remainder of sum / W), once per (window, channel) by the last of the
// window's row blocks to finish
// ---------------------------------------------------------------------------------------
constexpr int kSumRows = 128;
constexpr int kSumThreads = 256;

// colsum [nb][C] and ticket [nb][gridDim.x] are zero on entry and left zero on exit (the last row
// block of a (window, channel block) clears them after taking the means), so no launch clears them
__global__ void __launch_bounds__(kSumThreads)
colsum_kernel(const int16_t* __restrict__ raw, int64_t row_stride, const int32_t* __restrict__ chan, int C, int W,
              int NT, long long* __restrict__ colsum, int* __restrict__ ticket, float* __restrict__ mean) {
    __shared__ int s_last;
    const int b = blockIdx.z;
    const int r0 = blockIdx.y * kSumRows;
    const int r1 = min(W, r0 + kSumRows);
    const int64_t base = (int64_t)b * NT;
    const int c = blockIdx.x * kSumThreads + threadIdx.x;   // gridDim.x * kSumThreads >= C
    long long* cs = colsum + (int64_t)b * C + c;
    if (c < C) {
        const int src = chan ? chan[c] : c;
        int acc = 0;
        for (int r = r0; r < r1; ++r) acc += raw[(base + r) * row_stride + src];
        atomicAdd(reinterpret_cast<unsigned long long*>(cs), (unsigned long long)(long long)acc);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        int* tk = ticket + (int64_t)b * gridDim.x + blockIdx.x;
        s_last = atomicAdd(tk, 1) == (int)gridDim.y - 1;
        if (s_last) *tk = 0;
    }
    __syncthreads();
    if (s_last && c < C) {
        const long long sum = __ldcg(cs);   // every row block's sum is in L2 (fenced before its ticket)
        const long long q = sum / W;        // |q| <= 32768: exact in FP32
        const int r = (int)(sum - q * W);   // |r| < W
        mean[(int64_t)b * C + c] = (float)q + __fdiv_rn((float)r, (float)W);
        *cs = 0;
    }
}

// The same sums with 16-byte loads, when the channels are the row's first C values (no channel
// map), C % 8 == 0 and rows start 16-byte aligned: thread (g, p) of a block adds channels
// 8g .. 8g+7 over the block's rows r = p (mod P), P = 256 / (C / 8); the P partial sums of a channel
// group are added in shared memory in p order, then one 64-bit atomic per channel; one ticket per
// window (the last row block takes the means).
constexpr int kSumRowsV = 64;
__global__ void __launch_bounds__(kSumThreads)
colsum_vec_kernel(const int16_t* __restrict__ raw, int64_t row_stride, int C, int W, int NT,
                  long long* __restrict__ colsum, int* __restrict__ ticket, float* __restrict__ mean) {
    extern __shared__ int s_part[];   // [P][C]
    __shared__ int s_last;
    const int b = blockIdx.y;
    const int r0 = blockIdx.x * kSumRowsV, r1 = min(W, r0 + kSumRowsV);
    const int CG = C >> 3, P = kSumThreads / CG;
    const int g = threadIdx.x % CG, p = threadIdx.x / CG;
    if (p < P) {
        int acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        const int16_t* base = raw + (int64_t)b * NT * row_stride + 8 * g;
        for (int r = r0 + p; r < r1; r += P) {
            const uint4 v = __ldcs(reinterpret_cast<const uint4*>(base + (int64_t)r * row_stride));
            const uint32_t u[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                acc[2 * e] += (int)(int16_t)(u[e] & 0xffffu);
                acc[2 * e + 1] += (int)(int16_t)(u[e] >> 16);
            }
        }
#pragma unroll
        for (int e = 0; e < 8; ++e) s_part[p * C + 8 * g + e] = acc[e];
    }
    __syncthreads();
    long long* cs = colsum + (int64_t)b * C;
    for (int c = threadIdx.x; c < C; c += kSumThreads) {
        int tot = 0;
        for (int q = 0; q < P; ++q) tot += s_part[q * C + c];
        atomicAdd(reinterpret_cast<unsigned long long*>(cs + c), (unsigned long long)(long long)tot);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        int* tk = ticket + b;
        s_last = atomicAdd(tk, 1) == (int)gridDim.x - 1;
        if (s_last) *tk = 0;
    }
    __syncthreads();
    if (s_last) {
        for (int c = threadIdx.x; c < C; c += kSumThreads) {
            const long long sum = __ldcg(cs + c);
            const long long q = sum / W;
            const int r = (int)(sum - q * W);
            mean[(int64_t)b * C + c] = (float)q + __fdiv_rn((float)r, (float)W);
            cs[c] = 0;
        }
    }
}

void launch_colsum(const int16_t* raw, int64_t row_stride, const int32_t* chan, int C, int W, int NT, int nb,
                   long long* colsum, int* ticket, float* mean, cudaStream_t s) {
    const bool vec = !chan && C % 8 == 0 && C / 8 <= kSumThreads && (row_stride * 2) % 16 == 0 &&
                     (reinterpret_cast<uintptr_t>(raw) & 15) == 0;
    if (vec) {
        const int P = kSumThreads / (C / 8);
        dim3 grid((W + kSumRowsV - 1) / kSumRowsV, nb);
        colsum_vec_kernel<<<grid, kSumThreads, sizeof(int) * P * C, s>>>(raw, row_stride, C, W, NT, colsum, ticket,
                                                                          mean);
        return;
    }
    dim3 grid((C + kSumThreads - 1) / kSumThreads, (W + kSumRows - 1) / kSumRows, nb);
    colsum_kernel<<<grid, kSumThreads, 0, s>>>(raw, row_stride, chan, C, W, NT, colsum, ticket, mean);
}

// ---------------------------------------------------------------------------------------
// mean removal + lower median across channels (torch.median semantics), one warp per row
// ---------------------------------------------------------------------------------------
// tf32 split of an fp32 value: hi = tf32(x) (round to nearest, ties away), lo = x - hi
__device__ __forceinline__ void tf32_split_(float x, float& hi, float& lo) {
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    hi = __uint_as_float(h);
    lo = x - hi;
}

constexpr int kCarWarps = 8;

// NJ = channels per lane (C <= 32 * NJ), so the selection loop runs over live registers only
template <int NJ>
__global__ void __launch_bounds__(kCarWarps * 32)
car_kernel(const int16_t* __restrict__ raw, int64_t row_stride, const int32_t* __restrict__ chan, int C, int W,
           int NT, const float* __restrict__ mean, int L, int R, float* __restrict__ Xw) {
    constexpr int kMaxChanPerLane = NJ;
    const int b = blockIdx.y;
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * kCarWarps + (threadIdx.x >> 5);
    if (w >= W) return;
    const int64_t rowp = ((int64_t)b * NT + w) * row_stride;
    const int nj = (C + 31) >> 5;
    float v[kMaxChanPerLane];
    uint32_t key[kMaxChanPerLane];
#pragma unroll
    for (int j = 0; j < kMaxChanPerLane; ++j) {
        const int c = lane + 32 * j;
        if (j < nj && c < C) {
            const float x = (float)raw[rowp + (chan ? chan[c] : c)] - mean[(int64_t)b * C + c];
            v[j] = x;
            key[j] = float_key(x);
        } else {
            v[j] = 0.f;
            key[j] = 0xffffffffu;   // sorts after every real value, never selected (k < C)
        }
    }
    const float med = key_float(warp_kth_smallest<kMaxChanPerLane>(key, (C - 1) >> 1));
    const int rows = W + L + R;
    float* xb = Xw + (int64_t)b * rows * C;
    const bool wrapL = (w >= W - L);   // also lands in the left pad
    const bool wrapR = (w < R);        // also lands in the right pad
#pragma unroll
    for (int j = 0; j < kMaxChanPerLane; ++j) {
        const int c = lane + 32 * j;
        if (j < nj && c < C) {
            const float y = v[j] - med;
            xb[(int64_t)(w + L) * C + c] = y;
            if (wrapL) xb[(int64_t)(w + L - W) * C + c] = y;
            if (wrapR) xb[(int64_t)(w + L + W) * C + c] = y;
        }
    }
}

// Channel-major variant for the tensor-core high-pass: a CTA takes 32 consecutive samples, each
// warp four of them (the same median selection as car_kernel), stages the results in shared
// memory and writes Xt[(b, c)][w + L] (+ the wrap copies) as coalesced runs of 32 samples per
// channel, tf32-split into (Xt_hi, Xt_lo); columns past W + L + R up to the row pitch are zeroed.
// OUT: 0 = tf32(x) alone, 1 = the tf32 split, 2 = the BF16 split (Xt_hi / Xt_lo viewed as bf16)
constexpr int kCarTRows = 32;

template <int NJ, int OUT>
__global__ void __launch_bounds__(kCarWarps * 32)
car_t_kernel(const int16_t* __restrict__ raw, int64_t row_stride, const int32_t* __restrict__ chan, int C, int W,
             int NT, const float* __restrict__ mean, int L, int R, int pitch, float* __restrict__ Xt_hi,
             float* __restrict__ Xt_lo) {
    constexpr bool LO = OUT != 0;
    extern __shared__ float s_y[];   // [kCarTRows][C + 1]
    const int b = blockIdx.y;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int w0 = blockIdx.x * kCarTRows;
    const int ld = C + 1;
    for (int rr = warp; rr < kCarTRows; rr += kCarWarps) {
        const int w = w0 + rr;
        if (w >= W) break;
        const int64_t rowp = ((int64_t)b * NT + w) * row_stride;
        float v[NJ];
        uint32_t key[NJ];
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            const int c = lane + 32 * j;
            if (c < C) {
                const float x = (float)raw[rowp + (chan ? chan[c] : c)] - mean[(int64_t)b * C + c];
                v[j] = x;
                key[j] = float_key(x);
            } else {
                v[j] = 0.f;
                key[j] = 0xffffffffu;
            }
        }
        const float med = key_float(warp_kth_smallest<NJ>(key, (C - 1) >> 1));
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            const int c = lane + 32 * j;
            if (c < C) s_y[rr * ld + c] = v[j] - med;
        }
    }
    __syncthreads();
    const int nrows = min(kCarTRows, W - w0);
    const int total = W + L + R;
    for (int idx = threadIdx.x; idx < kCarTRows * C; idx += blockDim.x) {
        const int c = idx / kCarTRows, rr = idx - c * kCarTRows;
        const int64_t rbase = ((int64_t)b * C + c) * pitch;
        if constexpr (OUT == 2) {
            __nv_bfloat16* bh = reinterpret_cast<__nv_bfloat16*>(Xt_hi);
            __nv_bfloat16* bl = reinterpret_cast<__nv_bfloat16*>(Xt_lo);
            if (rr < nrows) {
                const int w = w0 + rr;
                const float x = s_y[rr * ld + c];
                const __nv_bfloat16 h = __float2bfloat16_rn(x);
                const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
                bh[rbase + w + L] = h;
                bl[rbase + w + L] = l;
                if (w >= W - L) {
                    bh[rbase + w + L - W] = h;
                    bl[rbase + w + L - W] = l;
                }
                if (w < R) {
                    bh[rbase + w + L + W] = h;
                    bl[rbase + w + L + W] = l;
                }
            }
            if (blockIdx.x == 0 && rr < pitch - total) {
                bh[rbase + total + rr] = __float2bfloat16_rn(0.f);
                bl[rbase + total + rr] = __float2bfloat16_rn(0.f);
            }
            continue;
        }
        if (rr < nrows) {
            const int w = w0 + rr;
            float h, l;
            tf32_split_(s_y[rr * ld + c], h, l);
            // (the remainder is absent on the tier that feeds TF32 data to the tensor cores)
            Xt_hi[rbase + w + L] = h;
            if constexpr (LO) Xt_lo[rbase + w + L] = l;
            if (w >= W - L) {
                Xt_hi[rbase + w + L - W] = h;
                if constexpr (LO) Xt_lo[rbase + w + L - W] = l;
            }
            if (w < R) {
                Xt_hi[rbase + w + L + W] = h;
                if constexpr (LO) Xt_lo[rbase + w + L + W] = l;
            }
        }
        if (blockIdx.x == 0 && rr < pitch - total) {   // row padding read by the last tiles' band
            Xt_hi[rbase + total + rr] = 0.f;
            if constexpr (LO) Xt_lo[rbase + total + rr] = 0.f;
        }
    }
}

void launch_car_t(const int16_t* raw, int64_t row_stride, const int32_t* chan, int C, int W, int NT, int nb,
                  const float* mean, int L, int R, int pitch, float* Xt_hi, float* Xt_lo, cudaStream_t s,
                  bool bf16) {
    dim3 grid((W + kCarTRows - 1) / kCarTRows, nb);
    const int nj = (C + 31) / 32;
    const size_t smem = (size_t)kCarTRows * (C + 1) * sizeof(float);
#define LSS_CART(N)                                                                                        \
    do {                                                                                                   \
        if (bf16 && Xt_lo) {                                                                               \
            raise_smem_limit((const void*)car_t_kernel<N, 2>, smem);                                       \
            car_t_kernel<N, 2><<<grid, kCarWarps * 32, smem, s>>>(raw, row_stride, chan, C, W, NT, mean, \
                                                                  L, R, pitch, Xt_hi, Xt_lo);              \
        } else if (Xt_lo) {                                                                                \
            raise_smem_limit((const void*)car_t_kernel<N, 1>, smem);                                       \
            car_t_kernel<N, 1><<<grid, kCarWarps * 32, smem, s>>>(raw, row_stride, chan, C, W, NT, mean, \
                                                                  L, R, pitch, Xt_hi, Xt_lo);              \
        } else {                                                                                           \
            raise_smem_limit((const void*)car_t_kernel<N, 0>, smem);                                       \
            car_t_kernel<N, 0><<<grid, kCarWarps * 32, smem, s>>>(raw, row_stride, chan, C, W, NT, mean, \
                                                                  L, R, pitch, Xt_hi, nullptr);            \
        }                                                                                                  \
    } while (0)
    if (nj <= 4) LSS_CART(4);
    else if (nj <= 8) LSS_CART(8);
    else if (nj <= 12) LSS_CART(12);
    else if (nj <= 16) LSS_CART(16);
    else if (nj <= 24) LSS_CART(24);
    else LSS_CART(32);
#undef LSS_CART
}

void launch_car(const int16_t* raw, int64_t row_stride, const int32_t* chan, int C, int W, int NT, int nb,
                const float* mean, int L, int R, float* Xw, cudaStream_t s) {
    dim3 grid((W + kCarWarps - 1) / kCarWarps, nb);
    const int nj = (C + 31) / 32;
#define LSS_CAR(N) car_kernel<N><<<grid, kCarWarps * 32, 0, s>>>(raw, row_stride, chan, C, W, NT, mean, L, R, Xw)
    if (nj <= 4) LSS_CAR(4);
    else if (nj <= 8) LSS_CAR(8);
    else if (nj <= 12) LSS_CAR(12);
    else if (nj <= 16) LSS_CAR(16);
    else if (nj <= 24) LSS_CAR(24);
    else LSS_CAR(32);
#undef LSS_CAR
}

// ---------------------------------------------------------------------------------------
// tf32 split of an fp32 value: hi = tf32(x) (round to nearest, ties away), lo = x - hi
__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo) {
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    hi = __uint_as_float(h);
    lo = x - hi;
}

// circular high-pass: Y[w][c] = sum_j taps[j] * Xw[w + j][c]   (taps zero-padded to kHpChunk)
// With Ylo != nullptr the output is written as its tf32 split (Y = hi, Ylo = lo).
// CTA = 32 channels x 128 rows; a thread owns one channel and 32 consecutive rows; each
// chunk of 32 taps is applied from a shared-memory tile of 159 rows.
// ---------------------------------------------------------------------------------------
constexpr int kHpRows = 128;
constexpr int kHpRowsPerThread = 32;
constexpr int kHpChunk = 32;
constexpr int kHpTile = kHpRows + kHpChunk - 1;

__global__ void __launch_bounds__(128)
highpass_kernel(const float* __restrict__ Xw, int C, int W, int rows_in, const float* __restrict__ taps, int ntaps,
                float* __restrict__ Y, float* __restrict__ Ylo) {
    __shared__ float xs[kHpTile][32];
    __shared__ float ts[kHpChunk];
    const int b = blockIdx.z;
    const int c0 = blockIdx.y * 32;
    const int w0 = blockIdx.x * kHpRows;
    const int tc = threadIdx.x & 31;
    const int rg = threadIdx.x >> 5;   // 0..3
    const float* xb = Xw + (int64_t)b * rows_in * C;
    float acc[kHpRowsPerThread];
#pragma unroll
    for (int r = 0; r < kHpRowsPerThread; ++r) acc[r] = 0.f;

    for (int j0 = 0; j0 < ntaps; j0 += kHpChunk) {
        __syncthreads();
        for (int i = threadIdx.x; i < kHpTile * 32; i += blockDim.x) {
            const int rr = i >> 5, cc = i & 31;
            const int row = w0 + j0 + rr, ch = c0 + cc;
            xs[rr][cc] = (row < rows_in && ch < C) ? xb[(int64_t)row * C + ch] : 0.f;
        }
        if (threadIdx.x < kHpChunk) ts[threadIdx.x] = taps[j0 + threadIdx.x];
        __syncthreads();
        float xv[kHpRowsPerThread + kHpChunk - 1];
#pragma unroll
        for (int u = 0; u < kHpRowsPerThread + kHpChunk - 1; ++u) xv[u] = xs[rg * kHpRowsPerThread + u][tc];
#pragma unroll
        for (int jj = 0; jj < kHpChunk; ++jj) {
            const float t = ts[jj];
#pragma unroll
            for (int r = 0; r < kHpRowsPerThread; ++r) acc[r] = fmaf(t, xv[r + jj], acc[r]);
        }
    }
    const int ch = c0 + tc;
    if (ch >= C) return;
    float* yb = Y + (int64_t)b * W * C;
    float* lb = Ylo ? Ylo + (int64_t)b * W * C : nullptr;
#pragma unroll
    for (int r = 0; r < kHpRowsPerThread; ++r) {
        const int w = w0 + rg * kHpRowsPerThread + r;
        if (w < W) {
            if (lb) {
                float h, l;
                tf32_split(acc[r], h, l);
                yb[(int64_t)w * C + ch] = h;
                lb[(int64_t)w * C + ch] = l;
            } else {
                yb[(int64_t)w * C + ch] = acc[r];
            }
        }
    }
}

void launch_highpass(const float* Xw, int C, int W, int L, int R, const float* taps, int nb, float* Y,
                     cudaStream_t s, float* Ylo) {
    const int ntaps = L + R + 1;
    dim3 grid((W + kHpRows - 1) / kHpRows, (C + 31) / 32, nb);
    highpass_kernel<<<grid, 128, 0, s>>>(Xw, C, W, W + L + R, taps, ntaps, Y, Ylo);
}

// ---------------------------------------------------------------------------------------
// temporal basis convolution: Bpc[w][k][c] = sum_m wPCA[k][m] * Z[w + m - nt/2][c]
// ---------------------------------------------------------------------------------------
constexpr int kConvRows = 8;        // rows per thread
constexpr int kConvMaxK = 8;

// two fp32 fused multiply-adds per instruction: d.{x,y} = a.{x,y} * b.{x,y} + d.{x,y}, each
// rounded like fmaf
__device__ __forceinline__ void fma2(unsigned long long& d, unsigned long long a, unsigned long long b) {
    asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(d) : "l"(a), "l"(b));
}
__device__ __forceinline__ unsigned long long dup2(float x) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(x));
    return r;
}

// Specialised for the common (nt, K) with K even: the basis sits in shared memory as [nt][K] (pairs
// of components one 8-byte load apart), each thread owns one channel and kConvRows rows, and every
// tap multiplies the kConvRows inputs it meets in packed pairs (fma.rn.f32x2, two fmaf per
// instruction).  Taps are applied in ascending order, as in basis_conv_generic.
// HI_ONLY: store tf32(x) alone (the tier that feeds TF32 data to the tensor cores); otherwise the
// tf32 split when Blo is given, else the fp32 values
template <int NT_, int K_, bool HI_ONLY>
__global__ void __launch_bounds__(128)
basis_conv_x2(const float* __restrict__ Z, int C, int W, const float* __restrict__ wPCA, float* __restrict__ Bpc,
              float* __restrict__ Blo) {
    static_assert(K_ % 2 == 0, "pairs of components");
    constexpr int KP = K_ / 2;
    constexpr int R = kConvRows;
    constexpr int H = NT_ / 2;
    __shared__ __align__(16) float s_w[NT_ * K_];   // [m][k]
    for (int i = threadIdx.x; i < NT_ * K_; i += blockDim.x) {
        const int m = i / K_, k = i - m * K_;
        s_w[i] = __ldg(wPCA + k * NT_ + m);
    }
    __syncthreads();
    const int b = blockIdx.z;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int w0 = blockIdx.y * R;
    if (c >= C) return;
    const float* zb = Z + (int64_t)b * W * C + c;
    unsigned long long acc[R][KP];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int j = 0; j < KP; ++j) acc[r][j] = 0ull;
    unsigned long long xs[R + NT_ - 1];
#pragma unroll
    for (int u = 0; u < R + NT_ - 1; ++u) {
        const int row = w0 + u - H;
        xs[u] = dup2((row >= 0 && row < W) ? __ldg(zb + (int64_t)row * C) : 0.f);
    }
    const unsigned long long* wp = reinterpret_cast<const unsigned long long*>(s_w);
#pragma unroll
    for (int m = 0; m < NT_; ++m) {
        unsigned long long wv[KP];
#pragma unroll
        for (int j = 0; j < KP; ++j) wv[j] = wp[m * KP + j];
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int j = 0; j < KP; ++j) fma2(acc[r][j], xs[m + r], wv[j]);
    }
    float* ob = Bpc + (int64_t)b * W * K_ * C;
    float* lb = Blo ? Blo + (int64_t)b * W * K_ * C : nullptr;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int w = w0 + r;
        if (w < W) {
#pragma unroll
            for (int j = 0; j < KP; ++j) {
                const float2 v = *reinterpret_cast<const float2*>(&acc[r][j]);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float a = h ? v.y : v.x;
                    const int64_t o = ((int64_t)w * K_ + 2 * j + h) * C + c;
                    if constexpr (HI_ONLY) {
                        float hi, lo;
                        tf32_split(a, hi, lo);
                        ob[o] = hi;
                    } else if (lb) {
                        float hi, lo;
                        tf32_split(a, hi, lo);
                        ob[o] = hi;
                        lb[o] = lo;
                    } else {
                        ob[o] = a;
                    }
                }
            }
        }
    }
}

// Any (nt, K <= 8): basis read from global memory (cached).
__global__ void __launch_bounds__(128)
basis_conv_generic(const float* __restrict__ Z, int C, int W, const float* __restrict__ wPCA, int K, int nt,
                   float* __restrict__ Bpc, float* __restrict__ Blo, bool round_tf32) {
    const int b = blockIdx.z;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int w0 = blockIdx.y * kConvRows;
    if (c >= C) return;
    const float* zb = Z + (int64_t)b * W * C;
    const int H = nt / 2;
    float acc[kConvRows][kConvMaxK];
#pragma unroll
    for (int r = 0; r < kConvRows; ++r)
#pragma unroll
        for (int k = 0; k < kConvMaxK; ++k) acc[r][k] = 0.f;
    for (int u = 0; u < kConvRows + nt - 1; ++u) {
        const int row = w0 + u - H;
        const float x = (row >= 0 && row < W) ? __ldg(zb + (int64_t)row * C + c) : 0.f;
#pragma unroll
        for (int r = 0; r < kConvRows; ++r) {
            const int m = u - r;
            if (m >= 0 && m < nt) {
#pragma unroll
                for (int k = 0; k < kConvMaxK; ++k)
                    if (k < K) acc[r][k] = fmaf(x, __ldg(wPCA + k * nt + m), acc[r][k]);
            }
        }
    }
    float* ob = Bpc + (int64_t)b * W * K * C;
    float* lb = Blo ? Blo + (int64_t)b * W * K * C : nullptr;
#pragma unroll
    for (int r = 0; r < kConvRows; ++r) {
        const int w = w0 + r;
        if (w < W)
            for (int k = 0; k < K; ++k) {
                const int64_t o = ((int64_t)w * K + k) * C + c;
                if (lb || round_tf32) {
                    float h, l;
                    tf32_split(acc[r][k], h, l);
                    ob[o] = h;
                    if (lb) lb[o] = l;
                } else {
                    ob[o] = acc[r][k];
                }
            }
    }
}



// Host-side basis (needed for the parameter-bank specialisation).
void launch_basis_conv_host(const float* Z, int C, int W, const float* wPCA_dev, const float* wPCA_host, int K,
                            int nt, int nb, float* Bpc, cudaStream_t s, float* Blo, bool round_tf32) {
    dim3 grid((C + 127) / 128, (W + kConvRows - 1) / kConvRows, nb);
    (void)wPCA_host;
    if (nt == 61 && K == 6) {
        if (round_tf32 && !Blo)
            basis_conv_x2<61, 6, true><<<grid, 128, 0, s>>>(Z, C, W, wPCA_dev, Bpc, nullptr);
        else
            basis_conv_x2<61, 6, false><<<grid, 128, 0, s>>>(Z, C, W, wPCA_dev, Bpc, Blo);
    } else {
        basis_conv_generic<<<grid, 128, 0, s>>>(Z, C, W, wPCA_dev, K, nt, Bpc, Blo, round_tf32);
    }
}

}  // namespace lss
