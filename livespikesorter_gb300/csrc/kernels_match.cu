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
#include <climits>

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

constexpr int kVecSmem = 4;      // float4 per lane per pass of the subtraction (512 templates)
constexpr int kVecGlobal = 2;    // 256 templates: the global variant runs at 64 registers

// accepted spikes one iteration can hold in the shared list: the (2nt+1) max pool admits at most
// one per nt + 1 samples, twice that with exact ties; more fall back to reading the spike maps
__host__ __device__ inline int match_near_cap(int W, int nt) { return 2 * ((W + nt) / (nt + 1)) + 32; }

constexpr int kStageChunk = 4096;   // samples of per-sample maxima staged at once in B1

// dynamic shared memory of one CTA: [owned score rows if SMEM_B][cfmax of a window chunk + 2nt]
// [1/nm][nm][own samples' argmax][per-32-sample accepted masks and prefix]
// [two accepted-spike lists (sample, template, amp), by iteration parity]
__host__ __device__ inline size_t match_smem_bytes(int W, int T, int nt, int G, bool smem_b) {
    const size_t span = (size_t)(W + G - 1) / G;
    const size_t chunk = (size_t)(W < kStageChunk ? W : kStageChunk);
    const size_t pad = (chunk + 2 * nt + 3) & ~(size_t)3;   // 1/nm starts 16-byte aligned
    const size_t words = (size_t)(W + 31) / 32 + 1;
    return (smem_b ? span * T * 4 : 0) + pad * 4 + (size_t)T * 8 + span * 4 + words * 8 +
           2 * (size_t)match_near_cap(W, nt) * 12;
}

// shared::cluster address of the same shared variable in CTA `rank` of the cluster
__device__ __forceinline__ unsigned dsmem_addr(const void* local, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;"
                 : "=r"(r)
                 : "r"((unsigned)__cvta_generic_to_shared(local)), "r"(rank));
    return r;
}

// ctc is read by every batch (about 30 times per group launch from a table the size of L2) while
// the score rows stream through once per iteration: its lines are loaded, and prefetched, under an
// L2 evict-last policy so the score traffic evicts them last
__device__ __forceinline__ uint64_t l2_keep_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ float4 ld_keep(const float4* p, uint64_t pol) {
    float4 v;
    asm volatile("ld.global.nc.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p), "l"(pol));
    return v;
}

// One thread-block cluster (G CTAs) runs the matching loop of one batch.  CTA r owns the samples
// w = r, r + G, r + 2G, ... (interleaved, so the ~2nt+1 samples each spike touches spread evenly
// over the cluster instead of loading the one or two CTAs whose contiguous slice holds them).
// Per iteration:
//   B1  every CTA stages the whole window's per-sample maxima, tests its own samples (window max
//       over +-nt, threshold) and writes their accepted (template, amplitude) maps;
//   --  cluster barrier;
//   B2  every CTA reads the whole accepted map, ranks the spikes in sample order (the list is in
//       (iteration, sample) order), keeps them in a shared list and records its own;
//   C   each CTA subtracts amp * ctc from the score rows of its own samples within +-nt of a spike,
//       in ascending spike order, and recomputes those samples' maxima;
//   --  cluster barrier.
template <int G, bool SMEM_B, int NTHR>
__global__ void __launch_bounds__(NTHR, (SMEM_B || NTHR > 512) ? 1 : 2)
match_kernel(float* __restrict__ Bt, float* __restrict__ Xres, const float* __restrict__ ctcP,
             const float* __restrict__ pre_wf, const float* __restrict__ nm, float th2, int W, int T, int C,
             int nt, int max_iters, MatchScratch sc, MatchOut out) {
    constexpr int kWarps = NTHR / 32;
    constexpr int kVec = SMEM_B ? kVecSmem : kVecGlobal;
    extern __shared__ float smem[];
    const int b = blockIdx.x / G;
    const int rank = (G == 1) ? 0 : (int)cluster_rank();
    const int span = (W + G - 1) / G;
    const int own = rank < W ? (W - rank + G - 1) / G : 0;   // samples rank + G*j < W
    const int chunk = min(W, kStageChunk);
    const int nwords = (W + 31) / 32;
    const int near_cap = match_near_cap(W, nt);
    float* Bs = smem;                                                   // [span][T]: row j = sample rank + G*j
    float* s_cf = smem + (SMEM_B ? (size_t)span * T : 0);              // [chunk + 2nt]: cfmax of w at s_cf[w - c0 + nt]
    float* s_inm = s_cf + ((chunk + 2 * nt + 3) & ~3);                  // [T] 1 / nm, 16-byte aligned
    float* s_nm = s_inm + T;                                            // [T] nm
    int* s_imax = reinterpret_cast<int*>(s_nm + T);                     // [span] argmax of own sample j
    unsigned* s_mask = reinterpret_cast<unsigned*>(s_imax + span);      // [nwords + 1] accepted bits
    int* s_woff = reinterpret_cast<int*>(s_mask + nwords + 1);          // [nwords + 1] exclusive prefix
    // accepted-spike lists by iteration parity: the spikes of iteration it arrive unordered in
    // list it & 1 (sent by their owners into every CTA); the other list then holds them in sample
    // order for phase C
    int* s_lw = s_woff + nwords + 1;                                    // [2][near_cap] sample
    int* s_lt = s_lw + 2 * near_cap;                                    // [2][near_cap] template
    float* s_la = reinterpret_cast<float*>(s_lt + 2 * near_cap);        // [2][near_cap] amplitude
    __shared__ int s_wcnt[kWarps];
    __shared__ int s_lcnt[2];                                           // spikes received, by parity

    static_assert(G >= 2 && G <= 32, "one cluster of 2..32 CTAs per batch");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int L2 = 2 * nt + 1;
    const uint64_t pol_keep = l2_keep_policy();
    float* Bg = Bt + (int64_t)b * W * T;
    if (tid < 2) s_lcnt[tid] = 0;
    for (int q = tid; q <= nwords; q += NTHR) s_mask[q] = 0u;
    // score row of an own sample w = rank + G*j
    auto brow = [&](int w) -> float* { return SMEM_B ? Bs + (size_t)(w / G) * T : Bg + (int64_t)w * T; };
    float* cfmax = sc.cfmax + (int64_t)b * W;
    int* at_t = sc.at_t + (int64_t)b * W;
    float* at_amp = sc.at_amp + (int64_t)b * W;
    int* sp_w = out.sp_w + (int64_t)b * out.cap;
    int* sp_t = out.sp_t + (int64_t)b * out.cap;
    float* sp_amp = out.sp_amp + (int64_t)b * out.cap;
    int* sp_iter = out.sp_iter + (int64_t)b * out.cap;

    if (G > 1 && rank != (int)(blockIdx.x % G) && tid == 0) atomicOr(out.status + b, 2);
    if constexpr (SMEM_B) {
        // own rows, each contiguous in global memory
        const bool v4 = ((T & 3) == 0) && ((reinterpret_cast<uintptr_t>(Bg) & 15) == 0);
        const int per = v4 ? T / 4 : T;
        for (int64_t i = tid; i < (int64_t)own * per; i += NTHR) {
            const int j = (int)(i / per), e = (int)(i - (int64_t)j * per);
            const int64_t src = (int64_t)(rank + G * j) * T;
            if (v4)
                reinterpret_cast<float4*>(Bs + (size_t)j * T)[e] = __ldcs(reinterpret_cast<const float4*>(Bg + src) + e);
            else
                Bs[(size_t)j * T + e] = __ldcs(Bg + src + e);
        }
    }
    for (int t = tid; t < T; t += NTHR) {
        s_nm[t] = nm[t];
        s_inm[t] = 1.f / nm[t];
    }
    // a window of at most kStageChunk samples keeps every sample's maximum in every CTA: owners
    // push each new value into all CTAs, so phase B1 reads shared memory only
    const bool resident = W <= kStageChunk;
    if (resident)
        for (int i = tid; i < W + 2 * nt; i += NTHR)
            if (i < nt || i >= W + nt) s_cf[i] = -FLT_MAX;
    // every CTA of the cluster has started (and initialised its lists) before any writes into
    // another's shared memory
    group_barrier<G>();

    // warp-wide max / argmax of relu(x)^2 / nm (first index on ties) into cfmax / imax of w
    auto finish_sample = [&](int w, float best, int bi) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        const bool inner = w >= nt && w < W - nt;
        const float v = inner ? best : 0.f;
        if (lane == 0) {
            if (!resident) cfmax[w] = v;
            s_imax[w / G] = inner ? bi : 0;
        }
        if (resident && lane < G)
            asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(dsmem_addr(s_cf + w + nt, (unsigned)lane)), "f"(v)
                         : "memory");
    };

    // ---- A (once): per-sample max / argmax over templates of the own samples ----
    for (int j = warp; j < own; j += kWarps) {
        const int w = rank + G * j;
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

    const bool vec_ok = (T & 3) == 0 &&
                        ((reinterpret_cast<uintptr_t>(ctcP) | reinterpret_cast<uintptr_t>(Bt)) & 15) == 0;
    int n_total = 0, iters = 0;
    // The spike maps at_t / at_amp (read only when an iteration overflows the shared lists or the
    // rows are not float4-aligned) hold -1 at every sample not accepted in the current iteration.
    // A full pass writes every own sample's entry; otherwise only accepted samples are written and
    // their owners clear them again once the sorted list has replaced the maps.
    bool full = true;
    for (int it = 0; it < max_iters; ++it) {
        // ---- B1: window max and acceptance on the own samples, chunk by chunk ----
        for (int c0 = 0; c0 < W; c0 += chunk) {
            const int c1 = min(W, c0 + chunk);
            if (!resident) {
                for (int i = tid; i < c1 - c0 + 2 * nt; i += NTHR) {
                    const int w = c0 - nt + i;
                    s_cf[i] = (w >= 0 && w < W) ? __ldcg(cfmax + w) : -FLT_MAX;
                }
                __syncthreads();
            }
            // An accepted sample's own maximum is its window's maximum and above Th^2, so only
            // samples whose own maximum exceeds Th^2 are tested: the lanes screen 32 of the warp's
            // own samples (j = j0 + warp + kWarps*m) at once, then the whole warp takes each
            // candidate's window, lanes on consecutive maxima (own samples are G apart, so one
            // thread per window would hit the same banks).
            const int j0 = c0 > rank ? (c0 - rank + G - 1) / G : 0;
            const int j1 = c1 > rank ? min(own, (c1 - rank + G - 1) / G) : 0;   // own samples in [c0, c1)
            for (int m0 = 0; j0 + warp + kWarps * m0 < j1; m0 += 32) {
                const int js = j0 + warp + kWarps * (m0 + lane);
                const bool cand = js < j1 && s_cf[rank + G * js - c0 + nt] > th2;
                if (full && js < j1 && !cand) at_t[rank + G * js] = -1;
                unsigned cbits = __ballot_sync(0xffffffffu, cand);
                while (cbits) {
                    const int j = j0 + warp + kWarps * (m0 + __ffs(cbits) - 1);
                    cbits &= cbits - 1;
                    const int w = rank + G * j;
                    const float* win = s_cf + (w - c0);   // cfmax of w - nt .. w + nt
                    float cm = -FLT_MAX;
                    for (int d = lane; d < L2; d += 32) cm = fmaxf(cm, win[d]);
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) cm = fmaxf(cm, __shfl_xor_sync(0xffffffffu, cm, o));
                    int tt = -1;
                    float amp = 0.f;
                    if (lane == 0) {
                        if (cm > th2 && win[nt] == cm) {
                            tt = s_imax[j];
                            amp = brow(w)[tt] / s_nm[tt];
                            // phase C of every CTA reads rows of ctcP[tt]: start pulling the (2nt+1) x T
                            // slab into L2 now, a barrier ahead of use
                            if (((T * 4) & 15) == 0) {
                                const float* slab = ctcP + (int64_t)tt * L2 * T;
                                asm volatile("cp.async.bulk.prefetch.L2.global.L2::cache_hint [%0], %1, %2;" ::"l"(slab),
                                             "r"((uint32_t)(L2 * T * 4)), "l"(pol_keep)
                                             : "memory");
                            }
                            at_t[w] = tt;   // the maps serve the overflow paths
                            at_amp[w] = amp;
                        } else if (full) {
                            at_t[w] = -1;
                        }
                    }
                    tt = __shfl_sync(0xffffffffu, tt, 0);
                    amp = __shfl_sync(0xffffffffu, amp, 0);
                    if (tt >= 0 && sc.rs.bt0) {
                        // low-precision scores: the amplitude from the exact FP32 projection of the
                        // split data operand, 16-byte loads, every lane's loads in flight at once
                        const MatchRescore& rs = sc.rs;
                        const int64_t xr = ((int64_t)b * W + w) * rs.kc;
                        const uint4* xh = reinterpret_cast<const uint4*>(rs.x_hi + xr);
                        const uint4* xl = reinterpret_cast<const uint4*>(rs.x_lo + xr);
                        const float4* wr = reinterpret_cast<const float4*>(rs.wall3 + (int64_t)tt * rs.kc);
                        float acc = 0.f;
                        for (int v = lane; v < rs.kc / 8; v += 32) {
                            const uint4 h = __ldg(xh + v), l = __ldg(xl + v);
                            const float4 w0 = __ldg(wr + 2 * v), w1 = __ldg(wr + 2 * v + 1);
                            const uint32_t hh[4] = {h.x, h.y, h.z, h.w}, ll[4] = {l.x, l.y, l.z, l.w};
                            const float ww[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                const float a0 = __uint_as_float(hh[e] << 16) + __uint_as_float(ll[e] << 16);
                                const float a1 = __uint_as_float(hh[e] & 0xffff0000u) + __uint_as_float(ll[e] & 0xffff0000u);
                                acc = fmaf(ww[2 * e], a0, acc);
                                acc = fmaf(ww[2 * e + 1], a1, acc);
                            }
                        }
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                        const float b0 = __ldg(rs.bt0 + ((int64_t)b * W + w) * T + tt);
                        amp = (brow(w)[tt] + (acc - b0)) / s_nm[tt];
                        if (lane == 0) at_amp[w] = amp;
                    }
                    if (tt >= 0 && lane < G) {
                        // into list p of CTA `lane`: claim a slot there, then write the entry
                        const int p = it & 1;
                        unsigned slot;
                        asm volatile("atom.shared::cluster.add.u32 %0, [%1], 1;"
                                     : "=r"(slot)
                                     : "r"(dsmem_addr(&s_lcnt[p], (unsigned)lane))
                                     : "memory");
                        if ((int)slot < near_cap) {
                            const int e = p * near_cap + (int)slot;
                            asm volatile("st.shared::cluster.s32 [%0], %1;" ::"r"(dsmem_addr(s_lw + e, (unsigned)lane)), "r"(w)
                                         : "memory");
                            asm volatile("st.shared::cluster.s32 [%0], %1;" ::"r"(dsmem_addr(s_lt + e, (unsigned)lane)), "r"(tt)
                                         : "memory");
                            asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(dsmem_addr(s_la + e, (unsigned)lane)), "f"(amp)
                                         : "memory");
                        }
                    }
                }
            }
            if (!resident) __syncthreads();   // the next chunk overwrites s_cf
        }
        group_barrier<G>();

        // ---- B2: the accepted spikes of the whole window, ranked in sample order ----
        const int p = it & 1, q = p ^ 1;
        const int total = s_lcnt[p];   // every CTA received every spike: the same count everywhere
        if (total == 0) break;
        ++iters;
        const bool listed = total <= near_cap;
        // with the sorted list and float4 rows nothing reads the maps this iteration: owners clear
        // their accepted samples' entries as they place them
        const bool use_list = vec_ok && listed;
        auto place = [&](int w, int tt, float amp, int r) {
            s_lw[q * near_cap + r] = w;
            s_lt[q * near_cap + r] = tt;
            s_la[q * near_cap + r] = amp;
            const int slot = n_total + r;
            if (w % G == rank) {
                if (slot < out.cap) {
                    sp_w[slot] = w;
                    sp_t[slot] = tt;
                    sp_amp[slot] = amp;
                    sp_iter[slot] = it;
                }
                if (use_list) at_t[w] = -1;
            }
        };
        if (listed && total <= 32) {
            // a handful of spikes: one warp ranks them by sample with shuffles
            if (warp == 0) {
                const bool have = lane < total;
                const int w = have ? s_lw[p * near_cap + lane] : INT_MAX;
                int r = 0;
                for (int k = 0; k < total; ++k) r += __shfl_sync(0xffffffffu, w, k) < w;
                if (have) place(w, s_lt[p * near_cap + lane], s_la[p * near_cap + lane], r);
            }
        } else if (listed) {
            // rank = accepted samples before w: a bitmap of the received samples and its word prefix
            for (int i = tid; i < total; i += NTHR) {
                const int w = s_lw[p * near_cap + i];
                atomicOr(&s_mask[w >> 5], 1u << (w & 31));
            }
            __syncthreads();
            const int wpw = (nwords + kWarps - 1) / kWarps;
            const int qa = min(nwords, warp * wpw), qb = min(nwords, qa + wpw);
            int wcnt = 0;
            for (int qq = qa + lane; qq < qb; qq += 32) wcnt += __popc(s_mask[qq]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) wcnt += __shfl_xor_sync(0xffffffffu, wcnt, o);
            if (lane == 0) s_wcnt[warp] = wcnt;
            __syncthreads();
            if (lane == 0) {
                int off = 0;
                for (int i = 0; i < warp; ++i) off += s_wcnt[i];
                for (int qq = qa; qq < qb; ++qq) {
                    s_woff[qq] = off;
                    off += __popc(s_mask[qq]);
                }
            }
            __syncthreads();
            for (int i = tid; i < total; i += NTHR) {
                const int w = s_lw[p * near_cap + i];
                const int r = s_woff[w >> 5] + __popc(s_mask[w >> 5] & ((1u << (w & 31)) - 1u));
                place(w, s_lt[p * near_cap + i], s_la[p * near_cap + i], r);
            }
        } else {
            // more spikes than the lists hold: rank them from the global maps
            const int wpw = (nwords + kWarps - 1) / kWarps;
            const int qa = min(nwords, warp * wpw), qb = min(nwords, qa + wpw);
            int wcnt = 0;
            for (int qq = qa; qq < qb; ++qq) {
                const int w = 32 * qq + lane;
                const unsigned m = __ballot_sync(0xffffffffu, w < W && __ldcg(at_t + w) >= 0);
                if (lane == 0) s_mask[qq] = m;
                wcnt += __popc(m);
            }
            if (lane == 0) s_wcnt[warp] = wcnt;
            __syncthreads();
            int off = 0;
            for (int i = lane; i < warp; i += 32) off += s_wcnt[i];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) off += __shfl_xor_sync(0xffffffffu, off, o);
            for (int qq = qa; qq < qb; ++qq) {
                const unsigned m = s_mask[qq];
                const int w = 32 * qq + lane;
                const int slot = n_total + off + __popc(m & ((1u << lane) - 1u));
                if (((m >> lane) & 1u) && w % G == rank && slot < out.cap) {
                    sp_w[slot] = w;
                    sp_t[slot] = __ldcg(at_t + w);
                    sp_amp[slot] = __ldcg(at_amp + w);
                    sp_iter[slot] = it;
                }
                off += __popc(m);
            }
        }
        __syncthreads();
        // the bitmap starts empty next iteration; so does the list the next iteration's spikes
        // arrive in (nobody sends before the barrier that ends this iteration)
        if (!(listed && total <= 32))
            for (int qq = tid; qq <= nwords; qq += NTHR) s_mask[qq] = 0u;
        if (tid == 0) s_lcnt[q] = 0;
        const int* s_nw = s_lw + q * near_cap;
        const int* s_nt = s_lt + q * near_cap;
        const float* s_na = s_la + q * near_cap;

        // ---- C: subtract the accepted spikes from the own samples near them ----
        const int n_near = total;
        if (use_list) {
            // The warp's own samples j = warp, warp + kWarps, ... with their nearby spikes (runs of
            // the list in sample order) are consumed as (sample, spike) items, two per pass: two
            // spikes of one sample (applied in order on its row) or the last spike of one sample
            // and the next sample's first.  A row's maximum is taken in the pass of its last spike.
            int j = warp, k = 0, kend = 0;
            // lo = first spike at or after w - nt of the current sample w; samples only grow, so
            // it only moves forward
            int lo = 0;
            auto seek = [&]() {   // from sample j on, the next own sample with nearby spikes
                while (j < own) {
                    const int w = rank + G * j;
                    while (lo < n_near && s_nw[lo] < w - nt) ++lo;
                    if (lo == n_near) {
                        j = own;
                        return;
                    }
                    const int ws = s_nw[lo];
                    if (ws <= w + nt) {
                        int e = lo + 1;
                        while (e < n_near && s_nw[e] <= w + nt) ++e;
                        k = lo;
                        kend = e;
                        return;
                    }
                    // nothing within nt of w: on to the warp's first own sample at or after
                    // ws - nt (> w), the next j = warp (mod kWarps) from jt
                    const int jt = (ws - nt - rank + G - 1) / G;
                    j = jt + ((warp - jt) % kWarps + kWarps) % kWarps;
                }
            };
            seek();
            const int T4 = T >> 2;
            auto ctc_row = [&](int kk, int w) {
                return reinterpret_cast<const float4*>(ctcP + ((int64_t)s_nt[kk] * L2 + (w - s_nw[kk] + nt)) * T);
            };
            while (j < own) {
                const int wA = rank + G * j;
                const int kA = k;
                const bool twoA = k + 1 < kend;
                k += twoA ? 2 : 1;
                const bool lastA = k >= kend;
                if (lastA) {
                    j += kWarps;
                    seek();
                }
                int wB = -1, kB = -1;
                bool lastB = false;
                if (!twoA && j < own) {   // one spike of A: pair it with the next item
                    wB = rank + G * j;
                    kB = k;
                    k += 1;
                    lastB = k >= kend;
                    if (lastB) {
                        j += kWarps;
                        seek();
                    }
                }
                const bool hasB = kB >= 0;
                const float aA0 = s_na[kA], a1 = twoA ? s_na[kA + 1] : (hasB ? s_na[kB] : 0.f);
                const float4* c0 = ctc_row(kA, wA);
                const float4* c1 = twoA ? ctc_row(kA + 1, wA) : (hasB ? ctc_row(kB, wB) : c0);
                const bool has1 = twoA || hasB;
                float4* bA = reinterpret_cast<float4*>(brow(wA));
                float4* bB = reinterpret_cast<float4*>(hasB ? brow(wB) : brow(wA));
                float bestA = -1.f, bestB = -1.f;
                int biA = 0x7fffffff, biB = 0x7fffffff;
                for (int fb = 0; fb < T4; fb += 32 * kVec) {
                    float4 v0[kVec], v1[kVec], xa[kVec], xb[kVec];
                    // the ctc rows and, when the scores live in L2, the score rows in one batch of
                    // loads: one round trip per step instead of two
#pragma unroll
                    for (int jj = 0; jj < kVec; ++jj) {
                        const int f = fb + lane + 32 * jj;
                        const bool ok = f < T4;
                        v0[jj] = ok ? ld_keep(c0 + f, pol_keep) : make_float4(0.f, 0.f, 0.f, 0.f);
                        v1[jj] = (ok && has1) ? ld_keep(c1 + f, pol_keep) : make_float4(0.f, 0.f, 0.f, 0.f);
                        if constexpr (!SMEM_B) {
                            xa[jj] = ok ? bA[f] : make_float4(0.f, 0.f, 0.f, 0.f);
                            xb[jj] = (ok && hasB) ? bB[f] : make_float4(0.f, 0.f, 0.f, 0.f);
                        }
                    }
#pragma unroll
                    for (int jj = 0; jj < kVec; ++jj) {
                        const int f = fb + lane + 32 * jj;
                        if (f < T4) {
                            const int t = 4 * f;
                            float4 x = SMEM_B ? bA[f] : xa[jj];
                            x.x = fmaf(-aA0, v0[jj].x, x.x);
                            x.y = fmaf(-aA0, v0[jj].y, x.y);
                            x.z = fmaf(-aA0, v0[jj].z, x.z);
                            x.w = fmaf(-aA0, v0[jj].w, x.w);
                            if (twoA) {
                                x.x = fmaf(-a1, v1[jj].x, x.x);
                                x.y = fmaf(-a1, v1[jj].y, x.y);
                                x.z = fmaf(-a1, v1[jj].z, x.z);
                                x.w = fmaf(-a1, v1[jj].w, x.w);
                            }
                            bA[f] = x;
                            const float4 im = reinterpret_cast<const float4*>(s_inm)[f];
                            if (lastA) {
                                float r, v;
                                r = fmaxf(x.x, 0.f); v = r * r * im.x; if (v > bestA) { bestA = v; biA = t; }
                                r = fmaxf(x.y, 0.f); v = r * r * im.y; if (v > bestA) { bestA = v; biA = t + 1; }
                                r = fmaxf(x.z, 0.f); v = r * r * im.z; if (v > bestA) { bestA = v; biA = t + 2; }
                                r = fmaxf(x.w, 0.f); v = r * r * im.w; if (v > bestA) { bestA = v; biA = t + 3; }
                            }
                            if (hasB) {
                                float4 y = SMEM_B ? bB[f] : xb[jj];
                                y.x = fmaf(-a1, v1[jj].x, y.x);
                                y.y = fmaf(-a1, v1[jj].y, y.y);
                                y.z = fmaf(-a1, v1[jj].z, y.z);
                                y.w = fmaf(-a1, v1[jj].w, y.w);
                                bB[f] = y;
                                if (lastB) {
                                    float r, v;
                                    r = fmaxf(y.x, 0.f); v = r * r * im.x; if (v > bestB) { bestB = v; biB = t; }
                                    r = fmaxf(y.y, 0.f); v = r * r * im.y; if (v > bestB) { bestB = v; biB = t + 1; }
                                    r = fmaxf(y.z, 0.f); v = r * r * im.z; if (v > bestB) { bestB = v; biB = t + 2; }
                                    r = fmaxf(y.w, 0.f); v = r * r * im.w; if (v > bestB) { bestB = v; biB = t + 3; }
                                }
                            }
                        }
                    }
                }
                if (lastA) finish_sample(wA, bestA, biA);
                if (hasB && lastB) finish_sample(wB, bestB, biB);
            }
        } else {
            for (int j = warp; j < own; j += kWarps) {
                const int wp = rank + G * j;
                float* br = brow(wp);
                float best = -1.f;
                int bi = 0x7fffffff;
                bool touched = false;
                // general shapes or an overfull list: the 2nt+1 neighbours from the spike maps,
                // scalar rows
                int n_sp = 0;
                for (int e0 = 0; e0 < L2; e0 += 32) {
                    const int w2 = wp - nt + e0 + lane;
                    const bool hit = e0 + lane < L2 && w2 >= 0 && w2 < W && __ldcg(at_t + w2) >= 0;
                    n_sp += __popc(__ballot_sync(0xffffffffu, hit));
                }
                int done = 0;
                for (int e0 = 0; e0 < L2 && n_sp > 0; e0 += 32) {
                    const int w2l = wp - nt + e0 + lane;
                    const bool hit = e0 + lane < L2 && w2l >= 0 && w2l < W && __ldcg(at_t + w2l) >= 0;
                    unsigned m = __ballot_sync(0xffffffffu, hit);
                    while (m) {
                        const int ee = e0 + __ffs(m) - 1;
                        m &= m - 1;
                        ++done;
                        const bool last = done == n_sp;
                        const int w2 = wp - nt + ee;
                        const float a = __ldcg(at_amp + w2);
                        const float* c = ctcP + ((int64_t)__ldcg(at_t + w2) * L2 + (2 * nt - ee)) * T;
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
                if (touched) finish_sample(wp, best, bi);
            }
        }
        n_total += total;
        full = !use_list;     // the maps still hold this iteration's spikes: rewrite them all
        group_barrier<G>();   // the changed samples' maxima are read by every CTA in B1
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
// (in list order) into shared memory.  Then a warp holds one row (up to 512 channels per pass) in
// registers, finds the spikes that touch it in list order (32 list entries per ballot), applies
// them -- loading the next spike's waveform row while it applies the current one -- and stores
// the row once: each element sees the same fmaf sequence as a per-spike read-modify-write.
// ---------------------------------------------------------------------------------------------
constexpr int kResRows = 64;
constexpr int kResList = 1024;
constexpr int kResElems = 16;    // floats each lane holds per pass: 512 channels per warp

template <bool VEC>
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
    // more spikes near these rows than the shared list holds: walk the whole list in global memory
    const bool over = s_over != 0;
    const int cnt = over ? n : min(s_n, kResList);
    const int* lw = over ? sw : s_w;
    const int* lt = over ? st : s_t;
    const float* la = over ? sa : s_a;
    float* X = Xres + (int64_t)b * W * C;
    constexpr int kSpan = 32 * kResElems;
    // element e of a lane: channel c0 + 4 (lane + 32 (e / 4)) + e % 4 (float4 rows), else c0 + lane + 32 e
    auto chan = [&](int c0, int e) { return VEC ? c0 + 4 * (lane + 32 * (e >> 2)) + (e & 3) : c0 + lane + 32 * e; };
    auto load = [&](const float* row, int c0, float (&v)[kResElems]) {
        if constexpr (VEC) {
#pragma unroll
            for (int q = 0; q < kResElems / 4; ++q) {
                const int c = c0 + 4 * (lane + 32 * q);
                const float4 f = c < C ? *reinterpret_cast<const float4*>(row + c) : make_float4(0.f, 0.f, 0.f, 0.f);
                v[4 * q] = f.x;
                v[4 * q + 1] = f.y;
                v[4 * q + 2] = f.z;
                v[4 * q + 3] = f.w;
            }
        } else {
#pragma unroll
            for (int e = 0; e < kResElems; ++e) v[e] = chan(c0, e) < C ? row[chan(c0, e)] : 0.f;
        }
    };
    for (int w = r0 + warp; w < r1; w += 8) {
        float* xrow = X + (int64_t)w * C;
        for (int c0 = 0; c0 < C; c0 += kSpan) {
            // the next list entry (in list order) whose spike touches row w, or -1
            int k0 = -32;
            unsigned m = 0u;
            auto next_spike = [&]() -> int {
                for (;;) {
                    if (m) {
                        const int k = k0 + __ffs(m) - 1;
                        m &= m - 1u;
                        return k;
                    }
                    k0 += 32;
                    if (k0 >= cnt) return -1;
                    const int k = k0 + lane;
                    bool t = false;
                    if (k < cnt) {
                        const int dw = w - lw[k];
                        t = dw >= -hw && dw <= hw;
                    }
                    m = __ballot_sync(0xffffffffu, t);
                }
            };
            auto wrow = [&](int k) { return pre_wf + ((int64_t)lt[k] * nt + (w - lw[k] + hw)) * C; };
            int kc = next_spike();
            if (kc < 0) continue;   // no spike touches this row
            float xv[kResElems], wa[kResElems], wb[kResElems];
            load(xrow, c0, xv);
            load(wrow(kc), c0, wa);
            float aa = la[kc];
            while (kc >= 0) {
                const int kn = next_spike();
                float an = 0.f;
                if (kn >= 0) {
                    load(wrow(kn), c0, wb);
                    an = la[kn];
                }
#pragma unroll
                for (int e = 0; e < kResElems; ++e) xv[e] = fmaf(-aa, wa[e], xv[e]);
#pragma unroll
                for (int e = 0; e < kResElems; ++e) wa[e] = wb[e];
                aa = an;
                kc = kn;
            }
            if constexpr (VEC) {
#pragma unroll
                for (int q = 0; q < kResElems / 4; ++q) {
                    const int c = c0 + 4 * (lane + 32 * q);
                    if (c < C)
                        *reinterpret_cast<float4*>(xrow + c) =
                            make_float4(xv[4 * q], xv[4 * q + 1], xv[4 * q + 2], xv[4 * q + 3]);
                }
            } else {
#pragma unroll
                for (int e = 0; e < kResElems; ++e)
                    if (chan(c0, e) < C) xrow[chan(c0, e)] = xv[e];
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
                         const MatchOut& out, cudaStream_t s, int variant, bool residual) {
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
    if (e != cudaSuccess || !residual) return e;
    return launch_residual(Xres, pre_wf, out, W, C, nt, nb, s);
}

cudaError_t launch_residual(float* Xres, const float* pre_wf, const MatchOut& out, int W, int C, int nt, int nb,
                            cudaStream_t s) {
    dim3 grid((W + kResRows - 1) / kResRows, nb);
    const bool vec = (C & 3) == 0 && ((reinterpret_cast<uintptr_t>(Xres) | reinterpret_cast<uintptr_t>(pre_wf)) & 15) == 0;
    if (vec)
        residual_kernel<true><<<grid, 256, 0, s>>>(Xres, pre_wf, out, W, C, nt);
    else
        residual_kernel<false><<<grid, 256, 0, s>>>(Xres, pre_wf, out, W, C, nt);
    return cudaGetLastError();
}

}  // namespace lss
