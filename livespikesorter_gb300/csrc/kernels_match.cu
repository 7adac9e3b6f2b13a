// kernels_match.cu -- the matching-pursuit loop of Kilosort template_matching.py:157-198 as one
// persistent kernel per batch: a thread-block cluster of G CTAs owns one window, each CTA a
// contiguous slice of its time samples.  Per iteration:
//
//   A  per-sample max / argmax over templates of Cf = relu(B)^2 * (1/nm) (first and last nt
//      samples zeroed) -- computed for every sample before the loop, and afterwards only for
//      the samples phase C changed, by the warp that changed them, from the values it holds;
//   B1 (2nt+1) max pool of that per-sample max; accept a sample when the pooled value
//      exceeds Th^2 and equals the sample's own max; amplitude B[w][iY] / nm[iY];
//   B2 write the accepted spikes, ordered by (iteration, sample) like the reference;
//   C  subtract every accepted spike from the scores: B[w'][:] -= amp * ctc[:, iY, w'-w+nt] for
//      |w'-w| <= nt -- as a gather per output sample (each CTA updates only its own samples, so
//      no atomics and a fixed summation order).
//
// The loop never reads the residual, so the waveform subtraction Xres[w'][:] -= amp *
// waveform[iY][w'-w+nt/2] (|w'-w| <= nt/2) runs afterwards in residual_kernel, applying the
// spikes in the same (iteration, sample) order.
//
// When the CTA's slice of the score matrix fits (G = 16: ceil(W/16) samples x T templates x 4 B
// <= ~220 KB), it stays in shared memory for the whole loop; otherwise it is read and written in
// place in global memory (L2).  Phases are separated by hardware cluster barriers
// (barrier.cluster arrive.release / wait.acquire); data shared between CTAs goes through L2
// with .cg loads.  No spin-waits, no host round trips; the loop ends when an iteration accepts
// nothing (the same decision in every CTA) or after max_iters.
#include "lss_kernels.cuh"

#include <cfloat>

namespace lss {

template <int G>
__device__ __forceinline__ void group_barrier() {
    if constexpr (G == 1) {
        __syncthreads();
    } else {
        __syncthreads();
        asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
        asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
    }
}

__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
    return r;
}

constexpr int kMaxRoundsGlobal = 64;   // slice <= 64 * threads samples per CTA (scores in L2)
constexpr int kMaxRoundsSmem = 4;      // the shared-memory slice is at most a few hundred samples
constexpr int kPerLane = 8;      // row elements each lane loads before it stores (256 per warp)
constexpr int kNearMax = 128;    // spikes near one CTA's slice in one iteration (more: scalar path)
constexpr int kVecSmem = 4;      // float4 per lane per pass of the subtraction (512 templates)
constexpr int kVecGlobal = 2;    // 256 templates: the global variant runs at 64 registers

// dynamic shared memory of one CTA: [score slice if SMEM_B][s_cf][s_t][s_amp][1/nm], floats/ints
__host__ __device__ inline size_t match_smem_bytes(int W, int T, int nt, int G, bool smem_b) {
    const int span = (W + G - 1) / G;
    const size_t halo = (size_t)span + 2 * nt;
    // 1 / nm starts on a 16-byte boundary (read as float4)
    return (smem_b ? (size_t)span * T * 4 : 0) + ((halo * 3 + 3) & ~(size_t)3) * 4 + (size_t)T * 4;
}

template <int G, bool SMEM_B, int NTHR>
__global__ void __launch_bounds__(NTHR, (SMEM_B || NTHR > 512) ? 1 : 2)
match_kernel(float* __restrict__ Bt, float* __restrict__ Xres, const float* __restrict__ ctcP,
             const float* __restrict__ pre_wf, const float* __restrict__ nm, float th2, int W, int T, int C,
             int nt, int max_iters, MatchScratch sc, MatchOut out) {
    constexpr int kMatchThreads = NTHR;
    constexpr int kWarps = NTHR / 32;
    constexpr int kMaxRounds = SMEM_B ? kMaxRoundsSmem : kMaxRoundsGlobal;
    constexpr int kVec = SMEM_B ? kVecSmem : kVecGlobal;
    extern __shared__ float smem[];
    const int b = blockIdx.x / G;
    const int rank = (G == 1) ? 0 : (int)cluster_rank();
    const int span = (W + G - 1) / G;
    const int lo = min(W, rank * span), hi = min(W, lo + span);
    const int halo = span + 2 * nt;
    float* Bs = smem;                                                  // [span][T] when SMEM_B
    float* s_cf = smem + (SMEM_B ? (size_t)span * T : 0);            // [halo]
    int* s_t = reinterpret_cast<int*>(s_cf + halo);                    // [halo]
    float* s_amp = reinterpret_cast<float*>(s_t + halo);               // [halo]
    float* s_inm = s_cf + ((3 * halo + 3) & ~3);                      // [T] 1 / nm, 16-byte aligned
    __shared__ int s_cnt[G];
    __shared__ int s_woff[kMaxRounds * kWarps];
    __shared__ int s_total;
    __shared__ int s_nw[kNearMax], s_nt[kNearMax];
    __shared__ float s_na[kNearMax];
    __shared__ int s_nn;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int L2 = 2 * nt + 1;
    const int rounds = (hi - lo + kMatchThreads - 1) / kMatchThreads;
    float* Bg = Bt + (int64_t)b * W * T;
    // row pointer of sample w (own slice only)
    auto brow = [&](int w) -> float* { return SMEM_B ? Bs + (size_t)(w - lo) * T : Bg + (int64_t)w * T; };
    float* cfmax = sc.cfmax + (int64_t)b * W;
    int* imax = sc.imax + (int64_t)b * W;
    int* at_t = sc.at_t + (int64_t)b * W;
    float* at_amp = sc.at_amp + (int64_t)b * W;
    int* cta_cnt = sc.cta_cnt + (int64_t)b * 2 * G;
    int* sp_w = out.sp_w + (int64_t)b * out.cap;
    int* sp_t = out.sp_t + (int64_t)b * out.cap;
    float* sp_amp = out.sp_amp + (int64_t)b * out.cap;
    int* sp_iter = out.sp_iter + (int64_t)b * out.cap;

    if (G > 1 && rank != (int)(blockIdx.x % G) && tid == 0) atomicOr(out.status + b, 2);
    if (rounds > kMaxRounds && tid == 0) atomicOr(out.status + b, 2);
    if constexpr (SMEM_B) {
        // the slice [lo, hi) x T is contiguous in global memory
        const int64_t n = (int64_t)(hi - lo) * T;
        const float* src = Bg + (int64_t)lo * T;
        if ((((uintptr_t)src) & 15) == 0 && (n & 3) == 0) {
            const float4* s4 = reinterpret_cast<const float4*>(src);
            float4* d4 = reinterpret_cast<float4*>(Bs);
            for (int64_t i = tid; i < n / 4; i += kMatchThreads) d4[i] = __ldcs(s4 + i);
        } else {
            for (int64_t i = tid; i < n; i += kMatchThreads) Bs[i] = __ldcs(src + i);
        }
    }
    for (int t = tid; t < T; t += kMatchThreads) s_inm[t] = 1.f / nm[t];
    __syncthreads();

    // warp-wide max / argmax of relu(x)^2 / nm (first index on ties) into cfmax / imax of w
    auto finish_sample = [&](int w, float best, int bi) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (lane == 0) {
            const bool inner = w >= nt && w < W - nt;
            cfmax[w] = inner ? best : 0.f;
            imax[w] = inner ? bi : 0;
        }
    };

    // ---- A (once): per-sample max / argmax over templates of the whole slice ----
    for (int w = lo + warp; w < hi; w += kWarps) {
        const float* row = brow(w);
        float best = -1.f;
        int bi = 0x7fffffff;
        for (int t = lane; t < T; t += 32) {
            const float r = fmaxf(row[t], 0.f);
            const float v = r * r * s_inm[t];
            if (v > best) { best = v; bi = t; }
        }
        finish_sample(w, best, bi);
    }
    group_barrier<G>();

    int n_total = 0, iters = 0;
    for (int it = 0; it < max_iters && rounds <= kMaxRounds; ++it) {
        // ---- B1: pooled max and acceptance on the own slice; per-warp counts per round ----
        for (int i = tid; i < halo; i += kMatchThreads) {
            const int w = lo - nt + i;
            s_cf[i] = (w >= 0 && w < W) ? __ldcg(cfmax + w) : -FLT_MAX;
        }
        __syncthreads();
        for (int r = 0; r < rounds; ++r) {
            const int w = lo + r * kMatchThreads + tid;
            bool acc = false;
            if (w < hi) {
                const int i = w - lo + nt;
                float cm = -FLT_MAX;
                for (int d = -nt; d <= nt; ++d) cm = fmaxf(cm, s_cf[i + d]);
                const float cf = s_cf[i];
                int tt = -1;
                float amp = 0.f;
                if (cm > th2 && cf == cm) {
                    tt = imax[w];
                    amp = brow(w)[tt] / __ldg(nm + tt);
                    acc = true;
                    // phase C of every CTA near w reads rows of ctcP[tt]: start pulling the whole
                    // (2nt+1) x T slab into L2 now, a barrier and a few round trips ahead of use
                    if (((T * 4) & 15) == 0) {
                        const float* slab = ctcP + (int64_t)tt * L2 * T;
                        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(slab),
                                     "r"((uint32_t)(L2 * T * 4))
                                     : "memory");
                    }
                }
                at_t[w] = tt;
                at_amp[w] = amp;
            }
            const unsigned m = __ballot_sync(0xffffffffu, acc);
            if (lane == 0) s_woff[r * kWarps + warp] = __popc(m);
        }
        __syncthreads();
        if (tid == 0) {
            // exclusive prefix over (round, warp) = sample order within the slice
            int acc = 0;
            for (int i = 0; i < rounds * kWarps; ++i) {
                const int c = s_woff[i];
                s_woff[i] = acc;
                acc += c;
            }
            cta_cnt[(it & 1) * G + rank] = acc;
        }
        group_barrier<G>();

        // ---- totals: the same numbers in every CTA of the cluster ----
        if (tid < G) s_cnt[tid] = __ldcg(cta_cnt + (it & 1) * G + tid);
        __syncthreads();
        if (tid == 0) {
            int total = 0;
            for (int r = 0; r < G; ++r) total += s_cnt[r];
            s_total = total;
        }
        __syncthreads();
        const int total = s_total;
        if (total == 0) break;
        ++iters;
        int base = n_total;
        for (int r = 0; r < rank; ++r) base += s_cnt[r];

        // ---- B2: record the own slice's spikes in sample order (all threads) ----
        for (int r = 0; r < rounds; ++r) {
            const int w = lo + r * kMatchThreads + tid;
            const int tt = (w < hi) ? at_t[w] : -1;
            const unsigned m = __ballot_sync(0xffffffffu, tt >= 0);
            if (tt >= 0) {
                const int slot = base + s_woff[r * kWarps + warp] + __popc(m & ((1u << lane) - 1u));
                if (slot < out.cap) {
                    sp_w[slot] = w;
                    sp_t[slot] = tt;
                    sp_amp[slot] = at_amp[w];
                    sp_iter[slot] = it;
                }
            }
        }

        // ---- C: subtract the accepted spikes from the own samples ----
        for (int i = tid; i < halo; i += kMatchThreads) {
            const int w = lo - nt + i;
            const bool in = (w >= 0 && w < W);
            s_t[i] = in ? __ldcg(at_t + w) : -1;
            s_amp[i] = in ? __ldcg(at_amp + w) : 0.f;
        }
        __syncthreads();
        // the spikes near the own slice, in sample order (typically a handful): one compaction per
        // iteration instead of a scan of the 2nt+1 neighbours of every sample
        if (warp == 0) {
            int cnt = 0;
            for (int i0 = 0; i0 < halo; i0 += 32) {
                const int i = i0 + lane;
                const bool hit = i < halo && s_t[i] >= 0;
                const unsigned m = __ballot_sync(0xffffffffu, hit);
                if (hit) {
                    const int pos = cnt + __popc(m & ((1u << lane) - 1u));
                    if (pos < kNearMax) {
                        s_nw[pos] = lo - nt + i;
                        s_nt[pos] = s_t[i];
                        s_na[pos] = s_amp[i];
                    }
                }
                cnt += __popc(m);
            }
            if (lane == 0) s_nn = cnt;
        }
        __syncthreads();
        const int n_near = s_nn;
        const bool vec_ok = (T & 3) == 0 && n_near <= kNearMax && ((reinterpret_cast<uintptr_t>(ctcP) |
                                                                      reinterpret_cast<uintptr_t>(Bt)) & 15) == 0;
        for (int wp = lo + warp; wp < hi; wp += kWarps) {
            const int i0 = wp - lo;   // s_t[i0 + e] is the sample wp - nt + e
            float* br = brow(wp);
            float best = -1.f;
            int bi = 0x7fffffff;
            bool touched = false;
            if (vec_ok) {
                // spikes k with |w_k - wp| <= nt, two at a time, in sample order
                int k = 0;
                while (k < n_near) {
                    while (k < n_near && (s_nw[k] < wp - nt || s_nw[k] > wp + nt)) ++k;
                    if (k >= n_near) break;
                    int k2 = k + 1;
                    while (k2 < n_near && (s_nw[k2] < wp - nt || s_nw[k2] > wp + nt)) ++k2;
                    const bool two = k2 < n_near;
                    int k3 = two ? k2 + 1 : n_near;
                    while (k3 < n_near && (s_nw[k3] < wp - nt || s_nw[k3] > wp + nt)) ++k3;
                    const bool last = k3 >= n_near;   // no further spike for this sample
                    const float a0 = s_na[k], a1 = two ? s_na[k2] : 0.f;
                    const float4* c0 = reinterpret_cast<const float4*>(ctcP + ((int64_t)s_nt[k] * L2 + (wp - s_nw[k] + nt)) * T);
                    const float4* c1 = two ? reinterpret_cast<const float4*>(ctcP + ((int64_t)s_nt[k2] * L2 + (wp - s_nw[k2] + nt)) * T)
                                           : c0;
                    float4* b4 = reinterpret_cast<float4*>(br);
                    const int T4 = T >> 2;
                    for (int fb = 0; fb < T4; fb += 32 * kVec) {
                        float4 v0[kVec], v1[kVec];
#pragma unroll
                        for (int j = 0; j < kVec; ++j) {
                            const int f = fb + lane + 32 * j;
                            const bool ok = f < T4;
                            v0[j] = ok ? __ldg(c0 + f) : make_float4(0.f, 0.f, 0.f, 0.f);
                            v1[j] = (ok && two) ? __ldg(c1 + f) : make_float4(0.f, 0.f, 0.f, 0.f);
                        }
#pragma unroll
                        for (int j = 0; j < kVec; ++j) {
                            const int f = fb + lane + 32 * j;
                            if (f < T4) {
                                float4 x = b4[f];
                                x.x = fmaf(-a0, v0[j].x, x.x);
                                x.y = fmaf(-a0, v0[j].y, x.y);
                                x.z = fmaf(-a0, v0[j].z, x.z);
                                x.w = fmaf(-a0, v0[j].w, x.w);
                                if (two) {
                                    x.x = fmaf(-a1, v1[j].x, x.x);
                                    x.y = fmaf(-a1, v1[j].y, x.y);
                                    x.z = fmaf(-a1, v1[j].z, x.z);
                                    x.w = fmaf(-a1, v1[j].w, x.w);
                                }
                                b4[f] = x;
                                if (last) {
                                    const int t = 4 * f;
                                    const float4 im = reinterpret_cast<const float4*>(s_inm)[f];
                                    float r, v;
                                    r = fmaxf(x.x, 0.f); v = r * r * im.x; if (v > best) { best = v; bi = t; }
                                    r = fmaxf(x.y, 0.f); v = r * r * im.y; if (v > best) { best = v; bi = t + 1; }
                                    r = fmaxf(x.z, 0.f); v = r * r * im.z; if (v > best) { best = v; bi = t + 2; }
                                    r = fmaxf(x.w, 0.f); v = r * r * im.w; if (v > best) { best = v; bi = t + 3; }
                                }
                            }
                        }
                    }
                    touched = true;
                    k = two ? k2 + 1 : k + 1;
                }
            } else {
                // general shapes: scan the 2nt+1 neighbours, scalar rows
                int n_sp = 0;
                for (int e0 = 0; e0 < L2; e0 += 32) {
                    const int e = e0 + lane;
                    n_sp += __popc(__ballot_sync(0xffffffffu, e < L2 && s_t[i0 + e] >= 0));
                }
                int done = 0;
                for (int e0 = 0; e0 < L2 && n_sp > 0; e0 += 32) {
                    const int e = e0 + lane;
                    unsigned m = __ballot_sync(0xffffffffu, e < L2 && s_t[i0 + e] >= 0);
                    while (m) {
                        const int ee = e0 + __ffs(m) - 1;
                        m &= m - 1;
                        ++done;
                        const bool last = done == n_sp;
                        const float a = s_amp[i0 + ee];
                        const float* c = ctcP + ((int64_t)s_t[i0 + ee] * L2 + (2 * nt - ee)) * T;
                        for (int t = lane; t < T; t += 32) {
                            const float x = fmaf(-a, __ldg(c + t), br[t]);
                            br[t] = x;
                            if (last) {
                                const float r = fmaxf(x, 0.f);
                                const float v = r * r * s_inm[t];
                                if (v > best) { best = v; bi = t; }
                            }
                        }
                        touched = true;
                    }
                }
            }
            if (touched) finish_sample(wp, best, bi);
        }
        n_total += total;
        group_barrier<G>();   // cfmax of the changed samples is read by the neighbours in B1
    }
    if (rank == 0 && tid == 0) {
        out.n_spikes[b] = n_total;
        out.n_iters[b] = iters;
        if (n_total > out.cap) atomicOr(out.status + b, 1);
    }
}

// ---------------------------------------------------------------------------------------------
// residual: Xres[w][:] -= amp * waveform[t][w - w_s + nt/2][:] for every accepted spike with
// |w - w_s| <= nt/2, applied in list order = (iteration, sample) -- the order the reference's
// loop subtracts in.  A CTA owns kResRows rows; it first copies the spikes that can touch them
// (in list order) into shared memory, then each warp applies them to its rows.
// ---------------------------------------------------------------------------------------------
constexpr int kResRows = 64;
constexpr int kResList = 1024;

__global__ void __launch_bounds__(256)
residual_kernel(float* __restrict__ Xres, const float* __restrict__ pre_wf, MatchOut out, int W, int C, int nt) {
    __shared__ int s_w[kResList], s_t[kResList];
    __shared__ float s_a[kResList];
    __shared__ int s_n, s_over;
    const int b = blockIdx.y;
    const int r0 = blockIdx.x * kResRows, r1 = min(W, r0 + kResRows);
    const int hw = nt / 2;
    const int n = min(out.n_spikes[b], out.cap);
    const int* sw = out.sp_w + (int64_t)b * out.cap;
    const int* st = out.sp_t + (int64_t)b * out.cap;
    const float* sa = out.sp_amp + (int64_t)b * out.cap;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) { s_n = 0; s_over = 0; }
    __syncthreads();
    // order-preserving compaction of the spikes with r0 - hw <= w_s < r1 + hw
    for (int i0 = 0; i0 < n; i0 += blockDim.x) {
        const int i = i0 + threadIdx.x;
        const bool hit = i < n && sw[i] >= r0 - hw && sw[i] < r1 + hw;
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        __shared__ int s_wc[8];
        if (lane == 0) s_wc[warp] = __popc(m);
        __syncthreads();
        int before = s_n;
        for (int k = 0; k < warp; ++k) before += s_wc[k];
        if (hit) {
            const int pos = before + __popc(m & ((1u << lane) - 1u));
            if (pos < kResList) {
                s_w[pos] = sw[i];
                s_t[pos] = st[i];
                s_a[pos] = sa[i];
            } else {
                s_over = 1;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int tot = 0;
            for (int k = 0; k < 8; ++k) tot += s_wc[k];
            s_n += tot;
        }
        __syncthreads();
    }
    const bool over = s_over != 0;
    const int ns = min(s_n, kResList);
    float* X = Xres + (int64_t)b * W * C;
    for (int w = r0 + warp; w < r1; w += 8) {
        float* xrow = X + (int64_t)w * C;
        const int cnt = over ? n : ns;
        for (int k = 0; k < cnt; ++k) {
            const int ws = over ? sw[k] : s_w[k];
            const int dw = w - ws;
            if (dw < -hw || dw > hw) continue;
            const int ts = over ? st[k] : s_t[k];
            const float a = over ? sa[k] : s_a[k];
            const float* wrow = pre_wf + ((int64_t)ts * nt + (dw + hw)) * C;
            for (int c0 = 0; c0 < C; c0 += 32 * kPerLane) {
                float wv[kPerLane], xv[kPerLane];
#pragma unroll
                for (int j = 0; j < kPerLane; ++j) {
                    const int c = c0 + lane + 32 * j;
                    wv[j] = (c < C) ? __ldg(wrow + c) : 0.f;
                    xv[j] = (c < C) ? xrow[c] : 0.f;
                }
#pragma unroll
                for (int j = 0; j < kPerLane; ++j) {
                    const int c = c0 + lane + 32 * j;
                    if (c < C) xrow[c] = fmaf(-a, wv[j], xv[j]);
                }
            }
        }
    }
}

template <int G, bool SMEM_B, int NTHR>
static cudaError_t launch_match_cfg(float* Bt, float* Xres, const float* ctcP, const float* pre_wf, const float* nm,
                                    float th2, int W, int T, int C, int nt, int max_iters, int nb,
                                    const MatchScratch& sc, const MatchOut& out, cudaStream_t s) {
    const size_t smem = match_smem_bytes(W, T, nt, G, SMEM_B);
    auto kern = match_kernel<G, SMEM_B, NTHR>;
    cudaError_t e = raise_smem_limit((const void*)kern, smem);
    if (e != cudaSuccess) return e;
    if (G > 8) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nb * G, 1, 1);
    cfg.blockDim = dim3(NTHR, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = G;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, Bt, Xres, ctcP, pre_wf, nm, th2, W, T, C, nt, max_iters, sc, out);
}

// Can a cluster of 16 CTAs with the whole score slice in shared memory run on this device?
static int smem16_ok(int W, int T, int nt) {
    if ((W + 15) / 16 > kMaxRoundsSmem * kMatchThreadsSmem) return 0;
    const size_t smem = match_smem_bytes(W, T, nt, 16, true);
    int dev = 0, maxopt = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
    if (smem + 12288 > (size_t)maxopt) return 0;   // static shared memory and the driver reserve
    auto kern = match_kernel<16, true, kMatchThreadsSmem>;
    if (raise_smem_limit((const void*)kern, smem) != cudaSuccess ||
        cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16, 1, 1);
    cfg.blockDim = dim3(kMatchThreadsSmem, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 16;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// Can a cluster of 16 CTAs of 1024 threads (scores in L2, one CTA per SM) run on this device?
static int wide16_ok(int W, int T, int nt) {
    if ((W + 15) / 16 > kMaxRoundsGlobal * kMatchThreadsWide) return 0;
    const size_t smem = match_smem_bytes(W, T, nt, 16, false);
    auto kern = match_kernel<16, false, kMatchThreadsWide>;
    if (raise_smem_limit((const void*)kern, smem) != cudaSuccess ||
        cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16, 1, 1);
    cfg.blockDim = dim3(kMatchThreadsWide, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 16;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// 16 when the shared-memory variant fits, else 8; wide = the 16-CTA / 1024-thread global variant fits
int match_variant(int W, int T, int nt, bool* wide) {
    static thread_local int cW = -1, cT = -1, cnt = -1, cres = 0;
    static thread_local bool cwide = false;
    if (W != cW || T != cT || nt != cnt) {
        cres = smem16_ok(W, T, nt) > 0 ? 16 : 8;
        cwide = wide16_ok(W, T, nt) > 0;
        cW = W, cT = T, cnt = nt;
    }
    if (wide) *wide = cwide;
    return cres;
}

cudaError_t launch_match(float* Bt, float* Xres, const float* ctcP, const float* pre_wf, const float* nm, float th2,
                         int W, int T, int C, int nt, int max_iters, int nb, const MatchScratch& sc,
                         const MatchOut& out, cudaStream_t s, int variant) {
    // variant: 0 = automatic -- for groups of at most 8 batches (latency), scores in shared memory
    // when they fit, else in L2 with 16-CTA clusters of 1024 threads (one CTA per SM); larger
    // groups (throughput) scores in L2 with 8-CTA clusters, two CTAs per SM.  1 = the 8-CTA L2
    // variant, 2 = shared memory (falls back to 1 when it cannot launch), 3 = the 16-CTA L2
    // variant (falls back to 1)
    bool wide = false;
    const int fit = match_variant(W, T, nt, &wide);
    int kind = 1;
    if (variant == 2) kind = fit == 16 ? 2 : 1;
    else if (variant == 3) kind = wide ? 3 : 1;
    else if (variant == 0 && nb <= 8) kind = fit == 16 ? 2 : (wide ? 3 : 1);
    cudaError_t e;
    if (kind == 2)
        e = launch_match_cfg<16, true, kMatchThreadsSmem>(Bt, Xres, ctcP, pre_wf, nm, th2, W, T, C, nt, max_iters, nb,
                                                          sc, out, s);
    else if (kind == 3)
        e = launch_match_cfg<16, false, kMatchThreadsWide>(Bt, Xres, ctcP, pre_wf, nm, th2, W, T, C, nt, max_iters,
                                                           nb, sc, out, s);
    else
        e = launch_match_cfg<8, false, kMatchThreads>(Bt, Xres, ctcP, pre_wf, nm, th2, W, T, C, nt, max_iters, nb, sc,
                                                      out, s);
    if (e != cudaSuccess) return e;
    dim3 grid((W + kResRows - 1) / kResRows, nb);
    residual_kernel<<<grid, 256, 0, s>>>(Xres, pre_wf, out, W, C, nt);
    return cudaGetLastError();
}

}  // namespace lss
