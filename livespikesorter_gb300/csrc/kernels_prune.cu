// kernels_prune.cu -- the pruned matching tier: Kilosort's matching loop (template_matching.py:
// 157-198) restricted, at every sample, to the keep templates with the largest initial
// Cf = relu(B)^2 / nm.
//
// Kilosort scores every template at every sample in every iteration; almost all of those scores
// stay far below the threshold for the whole loop.  Here a selection kernel keeps, per sample,
// the templates that can plausibly win (the largest initial Cf; ties to the lower template id)
// with their scores, and the loop runs on those lists only: the per-sample maximum reads keep
// scores instead of T, and an accepted spike (w_s, t_s, amp) updates only the listed entries of
// the 2nt+1 samples around it, gathering ctc[t][t_s][w - w_s + nt] for each listed t.  A listed
// entry receives exactly the full loop's fmaf sequence (spikes applied in sample order), so the
// result equals the full loop's unless a template that is not listed at a sample would have won
// there after subtractions.
//
// Template numbers are the sorter's internal ones (by position along the probe), so the templates
// listed at one sample -- the ones overlapping the spikes near it -- have nearby numbers, and one
// warp (its lanes on the listed entries of one sample) reads a few neighbouring cache lines of one
// row of ctcP instead of one line per entry.
//
// Widened lists: a sample whose keep-th largest initial Cf is high (crowded -- a larger spike
// nearby outranks the templates a short list misses) lists keep_wide templates; the others list
// keep and mark the rest kListPad, which both loop forms skip.
//
// Layouts (device):
//   lrk   u16 [nb][W][KP]     listed templates of sample w, ascending (KP = kPruneKeepMax slots, keep used;
//                             kListPad past a short list)
//   lsc   f32 [nb][W][KP]     their running scores (initial B on entry), updated in place
//   ctcP  f32 [T][2nt+1][T]   ctcP[s][l][t] = ctc[t][s][l]
//
// The loop runs on a thread-block cluster per window where a CTA's share fits in shared memory
// (4 CTAs of 512 threads for groups, 8 for a few windows; each CTA owns every G-th sample and its
// first 16 list entries, the rest of a list staying in lsc), else on one CTA of 1024 threads per
// window with the per-sample maxima, the listed templates and their scores in shared memory as far
// as they fit (all three for windows up to ~1700 samples at 16 entries), the rest in global memory.
#include "lss_kernels.cuh"

#include <cfloat>
#include <climits>

namespace lss {

constexpr int kSelWarps = 8;
constexpr int KP = kPruneKeepMax;   // list slots per sample (32: one per lane)

// order-preserving key of a non-negative-or-padding float, inverted so the largest value has the
// smallest key
__device__ __forceinline__ uint32_t desc_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return ~((u & 0x80000000u) ? ~u : (u | 0x80000000u));
}

// The k-th smallest (0-based) of the warp's keys (n live ones; padding keys 0xffffffff), MSB first,
// one ballot-count per bit, stopping once a single key matches the prefix.
template <int NJ>
__device__ __forceinline__ uint32_t kth_key_bits(const uint32_t (&key)[NJ], int k, int alive) {
    uint32_t prefix = 0;
    for (int bit = 31; bit >= 0; --bit) {
        const uint32_t hi_mask = (bit == 31) ? 0u : (0xffffffffu << (bit + 1));
        int cnt = 0;
#pragma unroll
        for (int j = 0; j < NJ; ++j) cnt += ((key[j] & hi_mask) == prefix) && !((key[j] >> bit) & 1u);
        cnt = __reduce_add_sync(0xffffffffu, cnt);
        if (k >= cnt) {
            k -= cnt;
            prefix |= (1u << bit);
            alive -= cnt;
        } else {
            alive = cnt;
        }
        if (alive == 1) {
            const uint32_t m = 0xffffffffu << bit;
            uint32_t got = 0;
#pragma unroll
            for (int j = 0; j < NJ; ++j)
                if ((key[j] & m) == prefix) got = key[j];
            return __reduce_or_sync(0xffffffffu, got);
        }
    }
    return prefix;
}

// One warp per sample: the keep templates of largest Cf (ties: lower id), written in ascending
// order with their scores.  NJ = templates per lane (T <= 32 NJ); template t = lane + 32 j.
// The keep-th largest Cf is found by an MSB-first bitwise selection over the warp's keys (one
// ballot-count per bit, stopping once a single key matches the prefix); every key above it is
// taken, then the ties at it in ascending template order until keep are taken.
// Widened lists (keep_wide > keep): a crowded sample -- its keep-th largest Cf above crowd_cf --
// takes keep_wide templates by the same rule; the others take keep, their entries keep ..
// keep_wide-1 marked kListPad.
template <int NJ>
__global__ void __launch_bounds__(kSelWarps * 32)
prune_select_kernel(const float* __restrict__ Bt, const float* __restrict__ nm, int nb, int W, int T, int keep,
                    int keep_wide, float crowd_cf, uint16_t* __restrict__ lrk, float* __restrict__ lsc) {
    __shared__ float s_inm[32 * NJ];
    __shared__ uint32_t s_cand[kSelWarps * 64];
    __shared__ uint16_t s_cand_t[kSelWarps * 64];   // their templates (candidate order = template order)
    for (int t = threadIdx.x; t < T; t += kSelWarps * 32) s_inm[t] = 1.f / nm[t];   // as the loop computes it
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t g = (int64_t)blockIdx.x * kSelWarps + (threadIdx.x >> 5);
    if (g >= (int64_t)nb * W) return;
    const float* row = Bt + g * T;
    uint32_t key[NJ];
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
        const int t = lane + 32 * j;
        if (t < T) {
            const float r = fmaxf(__ldcs(row + t), 0.f);
            key[j] = desc_key(r * r * s_inm[t]);   // the loop's Cf, bit for bit
        } else {
            key[j] = 0xffffffffu;                         // after every real key (keep <= T)
        }
    }
    // the (keep - 1)-th smallest key.  Every lane's smallest key: the keep-th smallest of those 32
    // bounds it from above (keep lanes hold a key at or below it), so it is the (keep - 1)-th
    // smallest of the keys at or below that bound -- usually a few dozen, which the bitwise
    // selection then runs on (two per lane); otherwise it runs on all of them.
    uint32_t lmin = key[0];
#pragma unroll
    for (int j = 1; j < NJ; ++j) lmin = min(lmin, key[j]);
    uint32_t v = lmin;   // bitonic sort of the lane minima, ascending by lane
#pragma unroll
    for (int k2 = 2; k2 <= 32; k2 <<= 1)
#pragma unroll
        for (int j2 = k2 >> 1; j2 > 0; j2 >>= 1) {
            const uint32_t o = __shfl_xor_sync(0xffffffffu, v, j2);
            const bool up = ((lane & k2) == 0) == ((lane & j2) == 0);
            v = up ? min(v, o) : max(v, o);
        }
    const int kw = max(keep, keep_wide);   // the longest list a sample may take
    const uint32_t bound = __shfl_sync(0xffffffffu, v, kw - 1);
    int n_cand = 0;
#pragma unroll
    for (int j = 0; j < NJ; ++j) n_cand += key[j] <= bound;
    n_cand = __reduce_add_sync(0xffffffffu, n_cand);
    uint32_t prefix = 0, prefix_w = 0;
    if (n_cand <= 64) {
        uint32_t* cand = s_cand + (threadIdx.x >> 5) * 64;
        int base = 0;
        const uint32_t lt0 = (1u << lane) - 1u;
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            const bool c = key[j] <= bound;
            const unsigned m = __ballot_sync(0xffffffffu, c);
            if (c) {
                cand[base + __popc(m & lt0)] = key[j];
                s_cand_t[(threadIdx.x >> 5) * 64 + base + __popc(m & lt0)] = (uint16_t)(lane + 32 * j);
            }
            base += __popc(m);
        }
        __syncwarp();
        uint32_t ck[2];
        ck[0] = lane < n_cand ? cand[lane] : 0xffffffffu;
        ck[1] = lane + 32 < n_cand ? cand[lane + 32] : 0xffffffffu;
        __syncwarp();
        prefix = kth_key_bits<2>(ck, keep - 1, n_cand);
    } else {
        prefix = kth_key_bits<NJ>(key, keep - 1, 32 * NJ);
    }
    // crowded: the keep-th largest Cf (the key's value, Cf >= 0) above crowd_cf; only then the
    // kw-th key (the warp's decision: one sample per warp)
    const bool crowded = kw > keep && __uint_as_float(~prefix & 0x7fffffffu) > crowd_cf;
    if (crowded) {
        if (n_cand <= 64) {
            uint32_t* cand = s_cand + (threadIdx.x >> 5) * 64;
            uint32_t ck[2];
            ck[0] = lane < n_cand ? cand[lane] : 0xffffffffu;
            ck[1] = lane + 32 < n_cand ? cand[lane + 32] : 0xffffffffu;
            prefix_w = kth_key_bits<2>(ck, kw - 1, n_cand);
        } else {
            prefix_w = kth_key_bits<NJ>(key, kw - 1, 32 * NJ);
        }
    }
    const int cnt = crowded ? kw : keep;
    const uint32_t thr = crowded ? prefix_w : prefix;
    if (n_cand <= 64) {
        // the taken keys are all among the candidates (kept in template order): those before the
        // threshold, then its ties in template order until cnt, each written at its rank
        const uint32_t* cand = s_cand + (threadIdx.x >> 5) * 64;
        const uint16_t* cand_t = s_cand_t + (threadIdx.x >> 5) * 64;
        uint32_t ck[2];
        ck[0] = lane < n_cand ? cand[lane] : 0xffffffffu;
        ck[1] = lane + 32 < n_cand ? cand[lane + 32] : 0xffffffffu;
        const int below_c = __reduce_add_sync(0xffffffffu, (int)(ck[0] < thr) + (int)(ck[1] < thr));
        int ties_c = cnt - below_c, pos = 0;
        const uint32_t ltc = (1u << lane) - 1u;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const bool tie = ck[i] == thr;
            const unsigned tm = __ballot_sync(0xffffffffu, tie);
            const bool take = ck[i] < thr || (tie && __popc(tm & ltc) < ties_c);
            ties_c -= min(__popc(tm), max(ties_c, 0));
            const unsigned m = __ballot_sync(0xffffffffu, take);
            if (take) {
                const int t = cand_t[lane + 32 * i];
                const int64_t o = g * KP + pos + __popc(m & ltc);
                lrk[o] = (uint16_t)t;
                lsc[o] = row[t];
            }
            pos += __popc(m);
        }
        if (lane >= cnt && lane < kw) {
            lrk[g * KP + lane] = kListPad;
            lsc[g * KP + lane] = 0.f;
        }
        return;
    }
    int below = 0;   // keys strictly before the threshold (larger Cf): all taken
#pragma unroll
    for (int j = 0; j < NJ; ++j) below += key[j] < thr;
    below = __reduce_add_sync(0xffffffffu, below);
    int ties_left = cnt - below;
    // compaction of the taken templates into lanes 0..keep-1, in template order
    int pos = 0, my_t = -1;
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
        const bool tie = key[j] == thr;
        const unsigned tm = __ballot_sync(0xffffffffu, tie);
        const bool take_tie = tie && __popc(tm & lt) < ties_left;
        ties_left -= min(__popc(tm), max(ties_left, 0));
        const bool take = key[j] < thr || take_tie;
        const unsigned m = __ballot_sync(0xffffffffu, take);
        // the taken entry with index lane - pos among this j's taken lanes goes to this lane
        const int want = lane - pos;
        if (want >= 0 && want < __popc(m)) my_t = (int)__fns(m, 0u, want + 1) + 32 * j;   // its (want+1)-th set bit
        pos += __popc(m);
    }
    if (lane < cnt) {
        const int64_t o = g * KP + lane;
        lrk[o] = (uint16_t)my_t;
        lsc[o] = row[my_t];
    } else if (lane < kw) {
        const int64_t o = g * KP + lane;
        lrk[o] = kListPad;
        lsc[o] = 0.f;
    }
}

void launch_prune_select(const float* Bt, const float* nm, int nb, int W, int T, int keep, uint16_t* lrk, float* lsc,
                         cudaStream_t s, int keep_wide, float crowd_cf) {
    const int64_t warps = (int64_t)nb * W;
    const dim3 grid((unsigned)((warps + kSelWarps - 1) / kSelWarps));
    const int nj = (T + 31) / 32;
#define LSS_SEL(N) \
    prune_select_kernel<N><<<grid, kSelWarps * 32, 0, s>>>(Bt, nm, nb, W, T, keep, keep_wide, crowd_cf, lrk, lsc)
    if (nj <= 4) LSS_SEL(4);
    else if (nj <= 8) LSS_SEL(8);
    else if (nj <= 16) LSS_SEL(16);
    else LSS_SEL(32);
#undef LSS_SEL
}

// accepted spikes one iteration can hold: the (2nt+1) max pool admits one per nt + 1 samples,
// twice that with exact ties
__host__ __device__ inline int prune_iter_cap(int W, int nt) { return 2 * ((W + nt) / (nt + 1)) + 32; }

// dynamic shared memory: [1/nm: T f32][nm: T f32][unordered + sorted accepted lists: 2 x cap x 12 B,
// to 16 B], then the per-sample maxima [W + 2nt] f32, the max pool's block prefix and suffix
// maxima [2][W + 2nt] f32 and list slots [W] u8 when they fit, then the
// listed templates [W][ks] u16 when they fit as well, then their scores [W][ks] f32 (ks = keep
// rounded up to 8) when those fit too
__host__ __device__ inline size_t prune_smem_head(int T) { return ((size_t)T * 8 + 15) & ~(size_t)15; }
__host__ __device__ inline size_t prune_smem_fixed(int W, int T, int nt) {
    return prune_smem_head(T) + ((2 * (size_t)prune_iter_cap(W, nt) * 12 + 15) & ~(size_t)15);
}
// (per-sample maxima, the prefix and suffix block maxima of the max pool, list slots)
__host__ __device__ inline size_t prune_smem_cf(int W, int nt) {
    return (((size_t)(W + 2 * nt) * 12 + (size_t)W) + 15) & ~(size_t)15;
}
__host__ __device__ inline int prune_stride(int keep) { return (keep + 7) & ~7; }
__host__ __device__ inline size_t prune_smem_ranks(int W, int ks) { return ((size_t)W * ks * 2 + 15) & ~(size_t)15; }
__host__ __device__ inline size_t prune_smem_scores(int W, int ks) { return (size_t)W * ks * 4; }

constexpr int kItemsPerGroup = 8;   // samples a lane group updates at once (independent gathers in flight)

// One CTA per window.  Per iteration:
//   B1  every sample whose own maximum exceeds Th^2 and equals the maximum over +-nt is accepted
//       (Kilosort's rule, template_matching.py:172-173): the lanes screen 32 samples at once, then
//       the warp takes each candidate's window; template and amplitude come from the list slot of
//       the sample's maximum;
//   B2  the iteration's spikes are ranked by sample and appended to the output lists;
//   C   every sample within +-nt of a spike -- taken by the first spike (in sample order) whose
//       range covers it -- applies each covering spike in sample order to its listed scores (a
//       group of LPS lanes per sample, a lane per entry; 32 / LPS samples per warp at once) and
//       recomputes its maximum with a reduction over the group.
// mode bit 0: maxima and slots in shared memory (else cf_g / slot_g); bit 1: listed templates in
// shared memory (stride ks); bit 2: their scores as well (else in lsc_g, stride KP)
template <int NTHR, int LPS>
__global__ void __launch_bounds__(NTHR, 1)
match_pruned_kernel(const uint16_t* __restrict__ lrk_g, float* __restrict__ lsc_g, int keep,
                    const float* __restrict__ ctcP, const float* __restrict__ nm, float th2, int W, int T, int nt,
                    int max_iters, int mode, float* __restrict__ cf_g, unsigned char* __restrict__ slot_g,
                    MatchOut out) {
    constexpr int kWarps = NTHR / 32;
    constexpr int kGroups = 32 / LPS;            // samples a warp holds at once
    extern __shared__ __align__(16) unsigned char smraw[];
    const int b = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int gl = lane % LPS;                   // lane within its group = list entry
    const int grp = lane / LPS;                  // the warp's group
    const int L2 = 2 * nt + 1;
    const int cap_it = prune_iter_cap(W, nt);
    float* s_inm = reinterpret_cast<float*>(smraw);                     // [T]
    float* s_nm = s_inm + T;                                            // [T]
    int* s_aw = reinterpret_cast<int*>(smraw + prune_smem_head(T));     // [cap] accepted, unordered
    int* s_at = s_aw + cap_it;
    float* s_aa = reinterpret_cast<float*>(s_at + cap_it);
    int* s_sw = reinterpret_cast<int*>(s_aa + cap_it);                  // [cap] the same, by sample
    int* s_st = s_sw + cap_it;
    float* s_sa = reinterpret_cast<float*>(s_st + cap_it);
    __shared__ int s_cnt, s_over;

    // per-sample state: cfmax of w at cf[w + nt] (pads of nt at both ends) and the list slot of its
    // maximum; the listed templates RK[w][i] and their scores SC[w][i]
    unsigned char* next = smraw + prune_smem_fixed(W, T, nt);
    float* cf;
    float *pg = nullptr, *ph = nullptr;   // block prefix / suffix maxima of cf (shared-memory state only)
    unsigned char* slot;
    if (mode & 1) {
        cf = reinterpret_cast<float*>(next);
        pg = cf + (W + 2 * nt);
        ph = pg + (W + 2 * nt);
        slot = reinterpret_cast<unsigned char*>(ph + (W + 2 * nt));
        next += prune_smem_cf(W, nt);
    } else {
        cf = cf_g + (int64_t)b * (W + 2 * nt);
        slot = slot_g + (int64_t)b * W;
    }
    const uint16_t* rk_g = lrk_g + (int64_t)b * W * KP;
    float* sc_g = lsc_g + (int64_t)b * W * KP;
    const int ks = (mode & 2) ? prune_stride(keep) : KP;   // row stride of RK and SC
    const uint16_t* RK;
    float* SC;
    if (mode & 2) {
        uint16_t* r = reinterpret_cast<uint16_t*>(next);
        next += prune_smem_ranks(W, ks);
        float* sc = (mode & 4) ? reinterpret_cast<float*>(next) : nullptr;
        for (int q = tid; q < W * ks; q += NTHR) {
            const int w = q / ks, i = q - w * ks;
            r[q] = rk_g[(size_t)w * KP + i];
            if (sc) sc[q] = sc_g[(size_t)w * KP + i];
        }
        RK = r;
        SC = sc ? sc : sc_g;
    } else {
        RK = rk_g;
        SC = sc_g;
    }
    const int ss = (mode & 4) ? ks : KP;   // row stride of SC
    for (int t = tid; t < T; t += NTHR) {
        s_nm[t] = nm[t];
        s_inm[t] = 1.f / nm[t];
    }
    for (int i = tid; i < nt; i += NTHR) {
        cf[i] = -FLT_MAX;
        cf[W + nt + i] = -FLT_MAX;
    }
    if (tid == 0) {
        s_cnt = 0;
        s_over = 0;
    }
    __syncthreads();

    // the group's sample w, lane gl holding entry gl (score x, template r): Cf maximum over the list
    // (ties: lower template) into cf / slot
    auto finish = [&](int w, float x, int r, bool valid) {
        float best = -1.f;
        int bt = INT_MAX, bs = 0;
        if (valid && gl < keep && r != kListPad) {
            const float q = fmaxf(x, 0.f);
            best = q * q * s_inm[r];
            bt = r;
            bs = gl;
        }
#pragma unroll
        for (int o = LPS / 2; o > 0; o >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int ot = __shfl_xor_sync(0xffffffffu, bt, o);
            const int os = __shfl_xor_sync(0xffffffffu, bs, o);
            if (ob > best || (ob == best && ot < bt)) { best = ob; bt = ot; bs = os; }
        }
        if (valid && gl == 0) {
            const bool inner = w >= nt && w < W - nt;
            cf[w + nt] = inner ? best : 0.f;
            slot[w] = (unsigned char)bs;
        }
    };
    for (int w0 = warp * kGroups; w0 < W; w0 += kWarps * kGroups) {
        const int w = w0 + grp;
        const bool valid = w < W;
        const int r = valid && gl < keep ? RK[(size_t)w * ks + gl] : 0;
        const float x = valid && gl < keep ? SC[(size_t)w * ss + gl] : 0.f;
        finish(w, x, r, valid);
    }
    __syncthreads();

    int n_total = 0, iters = 0;
    int* sp_w = out.sp_w + (int64_t)b * out.cap;
    int* sp_t = out.sp_t + (int64_t)b * out.cap;
    float* sp_amp = out.sp_amp + (int64_t)b * out.cap;
    int* sp_iter = out.sp_iter + (int64_t)b * out.cap;
    for (int it = 0; it < max_iters; ++it) {
        // ---- B1: acceptance ----
        if (mode & 1) {
            // the (2nt+1) max pool of the padded maxima P = cf [W + 2nt] by blocks of L2 (van Herk /
            // Gil-Werman): pg[i] = max P[block start .. i], ph[i] = max P[i .. block end], and the
            // window of sample w, P[w .. w + 2nt], spans at most two blocks: max(ph[w], pg[w + 2nt])
            const int n = W + 2 * nt;
            for (int blk = warp; blk * L2 < n; blk += kWarps) {
                const int b0 = blk * L2, b1 = min(n, b0 + L2);
                float carry = -FLT_MAX;
                for (int c0 = b0; c0 < b1; c0 += 32) {
                    const int i = c0 + lane;
                    float v = i < b1 ? cf[i] : -FLT_MAX;
#pragma unroll
                    for (int d = 1; d < 32; d <<= 1) {
                        const float o = __shfl_up_sync(0xffffffffu, v, d);
                        if (lane >= d) v = fmaxf(v, o);
                    }
                    v = fmaxf(v, carry);
                    if (i < b1) pg[i] = v;
                    carry = __shfl_sync(0xffffffffu, v, 31);
                }
                carry = -FLT_MAX;
                for (int c1 = b1; c1 > b0; c1 -= 32) {
                    const int i = c1 - 32 + lane;
                    float v = i >= b0 ? cf[i] : -FLT_MAX;
#pragma unroll
                    for (int d = 1; d < 32; d <<= 1) {
                        const float o = __shfl_down_sync(0xffffffffu, v, d);
                        if (lane + d < 32) v = fmaxf(v, o);
                    }
                    v = fmaxf(v, carry);
                    if (i >= b0) ph[i] = v;
                    carry = __shfl_sync(0xffffffffu, v, 0);
                }
            }
            __syncthreads();
            for (int w = tid; w < W; w += NTHR) {
                const float c = cf[w + nt];
                if (c > th2 && c == fmaxf(ph[w], pg[w + 2 * nt])) {
                    const int i = slot[w];
                    const int tt = RK[(size_t)w * ks + i];
                    const float amp = SC[(size_t)w * ss + i] / s_nm[tt];
                    const int q = atomicAdd(&s_cnt, 1);
                    if (q < cap_it) {
                        s_aw[q] = w;
                        s_at[q] = tt;
                        s_aa[q] = amp;
                    } else {
                        s_over = 1;
                    }
                }
            }
        } else
        for (int w0 = warp * 32; w0 < W; w0 += kWarps * 32) {
            const int wl = w0 + lane;
            unsigned m = __ballot_sync(0xffffffffu, wl < W && cf[wl + nt] > th2);
            while (m) {
                const int w = w0 + __ffs(m) - 1;
                m &= m - 1u;
                float cm = -FLT_MAX;
                for (int d = lane; d < L2; d += 32) cm = fmaxf(cm, cf[w + d]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) cm = fmaxf(cm, __shfl_xor_sync(0xffffffffu, cm, o));
                if (lane == 0 && cm > th2 && cf[w + nt] == cm) {
                    const int i = slot[w];
                    const int tt = RK[(size_t)w * ks + i];
                    const float amp = SC[(size_t)w * ss + i] / s_nm[tt];
                    const int q = atomicAdd(&s_cnt, 1);
                    if (q < cap_it) {
                        s_aw[q] = w;
                        s_at[q] = tt;
                        s_aa[q] = amp;
                    } else {
                        s_over = 1;
                    }
                }
            }
        }
        __syncthreads();
        const int total = min(s_cnt, cap_it);
        if (total == 0) break;
        ++iters;
        // ---- B2: rank by sample (samples are distinct), append to the output ----
        for (int k = tid; k < total; k += NTHR) {
            const int w = s_aw[k];
            int r = 0;
            for (int q = 0; q < total; ++q) r += s_aw[q] < w;
            s_sw[r] = w;
            s_st[r] = s_at[k];
            s_sa[r] = s_aa[k];
            const int o = n_total + r;
            if (o < out.cap) {
                sp_w[o] = w;
                sp_t[o] = s_at[k];
                sp_amp[o] = s_aa[k];
                sp_iter[o] = it;
            }
        }
        __syncthreads();
        if (tid == 0) s_cnt = 0;   // read again only after the barrier ending C
        // ---- C: subtract the spikes from the listed scores of the samples near them ----
        const int n_items = total * L2;
        constexpr int kPerWarp = kItemsPerGroup * kGroups;
        for (int q0 = warp * kPerWarp; q0 < n_items; q0 += kWarps * kPerWarp) {
            int wv[kItemsPerGroup], kv[kItemsPerGroup], rv[kItemsPerGroup];
            float xv[kItemsPerGroup], cv[kItemsPerGroup], cv2[kItemsPerGroup];
            bool two[kItemsPerGroup];
#pragma unroll
            for (int u = 0; u < kItemsPerGroup; ++u) {
                const int q = q0 + u * kGroups + grp;
                int w = -1, k = 0;
                if (q < n_items) {
                    k = q / L2;
                    w = s_sw[k] - nt + (q - k * L2);
                    // outside the window, or taken by an earlier spike's item
                    if (w < 0 || w >= W || (k > 0 && w <= s_sw[k - 1] + nt)) w = -1;
                }
                wv[u] = w;
                kv[u] = k;
                two[u] = w >= 0 && k + 1 < total && s_sw[k + 1] - nt <= w;   // a second spike covers w
                rv[u] = 0;
                xv[u] = 0.f;
                if (w >= 0 && gl < keep) {
                    rv[u] = RK[(size_t)w * ks + gl];
                    xv[u] = SC[(size_t)w * ss + gl];
                }
            }
            // the ctc entries of the owning spike and of a second covering spike, every item's loads
            // in flight together
#pragma unroll
            for (int u = 0; u < kItemsPerGroup; ++u) {
                cv[u] = cv2[u] = 0.f;
                if (wv[u] >= 0 && gl < keep && rv[u] != kListPad) {
                    const int k = kv[u];
                    cv[u] = __ldg(ctcP + ((int64_t)s_st[k] * L2 + (wv[u] - s_sw[k] + nt)) * T + rv[u]);
                    if (two[u]) cv2[u] = __ldg(ctcP + ((int64_t)s_st[k + 1] * L2 + (wv[u] - s_sw[k + 1] + nt)) * T + rv[u]);
                }
            }
            // new scores, applied in sample order, and each lane's (Cf, template, slot) key: the
            // largest Cf wins, then the lower template (Cf >= 0, so its bits order like the values)
            unsigned long long key[kItemsPerGroup];
#pragma unroll
            for (int u = 0; u < kItemsPerGroup; ++u) {
                const int w = wv[u];
                key[u] = 0ull;
                if (w < 0) continue;
                const int k = kv[u];
                float x = fmaf(-s_sa[k], cv[u], xv[u]);
                if (two[u]) {
                    x = fmaf(-s_sa[k + 1], cv2[u], x);
                    for (int kk = k + 2; kk < total && s_sw[kk] - nt <= w; ++kk) {   // rare: a third
                        const float c = gl < keep && rv[u] != kListPad
                                            ? __ldg(ctcP + ((int64_t)s_st[kk] * L2 + (w - s_sw[kk] + nt)) * T + rv[u])
                                            : 0.f;
                        x = fmaf(-s_sa[kk], c, x);
                    }
                }
                if (gl < keep && rv[u] != kListPad) {
                    SC[(size_t)w * ss + gl] = x;
                    const float qv = fmaxf(x, 0.f);
                    const float cfv = qv * qv * s_inm[rv[u]];
                    key[u] = ((unsigned long long)__float_as_uint(cfv) << 32) |
                             ((unsigned long long)(0xffffu - (unsigned)rv[u]) << 8) | (unsigned)gl;
                }
            }
#pragma unroll
            for (int o = LPS / 2; o > 0; o >>= 1)
#pragma unroll
                for (int u = 0; u < kItemsPerGroup; ++u) {
                    const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key[u], o);
                    key[u] = ok > key[u] ? ok : key[u];
                }
#pragma unroll
            for (int u = 0; u < kItemsPerGroup; ++u) {
                const int w = wv[u];
                if (w >= 0 && gl == 0) {
                    const bool inner = w >= nt && w < W - nt;
                    cf[w + nt] = inner ? __uint_as_float((unsigned)(key[u] >> 32)) : 0.f;
                    slot[w] = (unsigned char)(key[u] & 0xffu);
                }
            }
        }
        n_total += total;
        __syncthreads();
    }
    if (tid == 0) {
        out.n_spikes[b] = n_total;
        out.n_iters[b] = iters;
        if (n_total > out.cap || s_over) atomicOr(out.status + b, 1);
    }
}

// ---------------------------------------------------------------------------------------------
// The same loop on a thread-block cluster of G CTAs per window, for windows whose per-sample state
// fits in shared memory.  CTA r owns the samples w = r, r + G, r + 2G, ... (interleaved, so the
// 2nt + 1 samples around a spike spread over the whole cluster): their listed templates and
// scores.  Every CTA keeps a replica of every sample's maximum Cf and of the template and score
// behind it; an owner pushes the new values of the samples it updates into all G CTAs through
// distributed shared memory.  So every CTA finds the same accepted spikes (max pool, threshold)
// and ranks them the same way on its own, and phase C updates the own samples near them.  Two
// cluster barriers per iteration: one between the acceptance and the first push (its arrival
// and wait split around the ranking), so that no CTA's replica changes while it is read, and one
// after phase C, so that every replica is whole before the next max pool.
// ---------------------------------------------------------------------------------------------
template <int G>
__device__ __forceinline__ void cluster_sync_all() {
    __syncthreads();
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
// the two halves of a cluster barrier, for local work between them
__device__ __forceinline__ void cluster_arrive() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
__device__ __forceinline__ unsigned prune_cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned prune_dsmem(const void* local, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"((unsigned)__cvta_generic_to_shared(local)), "r"(rank));
    return r;
}

constexpr int kClItems = 2;   // samples a lane group of the cluster form updates at once (2, 3, 4 measured: 2 best)

// shared memory of one CTA: [1/nm, nm: 2T f32][accepted lists: 6 x cap][own-item starts and
// prefix: 2 x (cap + 1) int], to 16 B; [cf, block prefix, block suffix: 3 (W + 2nt) f32][winner
// score W f32][winner template W i32][own lists: span x ks u16, to 16 B][own scores: span x ks f32]
// [the iteration's items: sample and spike, 2 x span i32]
__host__ __device__ inline size_t prune_cl_fixed(int W, int T, int nt) {
    const size_t cap = (size_t)prune_iter_cap(W, nt);
    return ((size_t)T * 8 + cap * 24 + (cap + 1) * 8 + cap * 4 + 15) & ~(size_t)15;
}
// the cluster form's lane groups: 16 lanes, one list entry each in shared memory; entries 16 and
// up (24- or 32-entry lists, or widened lists at crowded samples) stay in the global lists, so the
// shared-memory footprint -- and the L1 left for the ctc gathers -- is the 16-entry one
constexpr int kClLanes = 16;
__host__ __device__ inline size_t prune_cl_smem(int W, int T, int nt, int keep, int G) {
    const size_t span = (size_t)(W + G - 1) / G;
    const size_t ks = (size_t)prune_stride(keep < kClLanes ? keep : kClLanes);
    size_t b = prune_cl_fixed(W, T, nt);
    b += (size_t)(W + 2 * nt) * 12 + (size_t)W * 8;
    b += (span * ks * 2 + 15) & ~(size_t)15;
    return b + span * ks * 4 + span * 8 + span;
}

// EPL: list entries per lane (entry e = gl + LPS h, h < EPL), so 24 or 32 entries run on lane
// groups of 16 -- two samples per warp, as at 16 entries -- instead of groups of 32
template <int G, int NTHR, int LPS, int EPL>
__global__ void __launch_bounds__(NTHR, 2)
match_pruned_cluster_kernel(const uint16_t* __restrict__ lrk_g, float* __restrict__ lsc_g, int keep,
                            const float* __restrict__ ctcP, const float* __restrict__ nm, float th2, int W, int T,
                            int nt, int max_iters, MatchOut out) {
    constexpr int kWarps = NTHR / 32;
    constexpr int kGroups = 32 / LPS;
    constexpr int kItems = kClItems;              // samples a lane group updates at once
    static_assert(G <= LPS, "the lanes of a group push one CTA each");
    static_assert(LPS * EPL <= KP && kItems >= 1, "entries per group");
    static_assert(LPS == kClLanes, "shared-memory list width");
    extern __shared__ __align__(16) unsigned char smraw[];
    const int b = blockIdx.x / G;
    const int rank = (int)prune_cluster_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int gl = lane % LPS, grp = lane / LPS;
    const int L2 = 2 * nt + 1, n = W + 2 * nt;
    const int cap_it = prune_iter_cap(W, nt);
    const int span = (W + G - 1) / G;
    const int own = rank < W ? (W - rank + G - 1) / G : 0;
    const int ks = prune_stride(min(keep, LPS));   // shared-memory list stride: entries < LPS
    float* s_inm = reinterpret_cast<float*>(smraw);
    float* s_nm = s_inm + T;
    int* s_aw = reinterpret_cast<int*>(s_nm + T);
    int* s_at = s_aw + cap_it;
    float* s_aa = reinterpret_cast<float*>(s_at + cap_it);
    int* s_sw = reinterpret_cast<int*>(s_aa + cap_it);
    int* s_st = s_sw + cap_it;
    float* s_sa = reinterpret_cast<float*>(s_st + cap_it);
    int* s_lo = reinterpret_cast<int*>(s_sa + cap_it);     // [cap + 1] first own sample of spike k's items
    int* s_pre = s_lo + cap_it + 1;                        // [cap + 1] own items before spike k
    int* s_cb = s_pre + cap_it + 1;                        // [cap] ctcP offset of spike k's rows, less w T
    unsigned char* next = smraw + prune_cl_fixed(W, T, nt);
    float* cf = reinterpret_cast<float*>(next);            // [n] maximum of w at cf[w + nt]
    float* pg = cf + n;
    float* ph = pg + n;
    float* wsc = ph + n;                                   // [W] score behind cf
    int* wt = reinterpret_cast<int*>(wsc + W);             // [W] template behind cf
    uint16_t* RK = reinterpret_cast<uint16_t*>(wt + W);    // [span][ks] own lists
    float* SC = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(RK) +
                                         ((((size_t)span * ks * 2) + 15) & ~(size_t)15));   // [span][ks]
    int* s_itw = reinterpret_cast<int*>(SC + (size_t)span * ks);   // [span] item q's own sample
    int* s_itk = s_itw + span;                                     // [span] and the spike that takes it
    unsigned char* s_wide = reinterpret_cast<unsigned char*>(s_itk + span);   // [span] entries >= LPS in use
    __shared__ int s_cnt, s_over;

    const uint16_t* rk_g = lrk_g + (int64_t)b * W * KP;
    float* sc_g = lsc_g + (int64_t)b * W * KP;   // entries >= LPS are read and updated here
    for (int q = tid; q < own * ks; q += NTHR) {
        const int j = q / ks, i = q - j * ks;
        const int w = rank + G * j;
        RK[q] = i < keep ? rk_g[(size_t)w * KP + i] : (uint16_t)0;
        SC[q] = i < keep ? sc_g[(size_t)w * KP + i] : 0.f;
    }
    for (int j = tid; j < own; j += NTHR)
        s_wide[j] = keep > LPS && rk_g[(size_t)(rank + G * j) * KP + LPS] != kListPad;
    for (int t = tid; t < T; t += NTHR) {
        s_nm[t] = nm[t];
        s_inm[t] = 1.f / nm[t];
    }
    for (int i = tid; i < nt; i += NTHR) {
        cf[i] = -FLT_MAX;
        cf[W + nt + i] = -FLT_MAX;
    }
    if (tid == 0) {
        s_cnt = 0;
        s_over = 0;
    }
    // every CTA of the cluster has started before any pushes into another's shared memory
    cluster_sync_all<G>();

    // this layout in CTA gl of the cluster (the lanes gl < G of a group push into CTA gl): the same
    // offsets from its shared-memory window
    const unsigned sm_base = (unsigned)__cvta_generic_to_shared(smraw);
    const unsigned rem = gl < G ? prune_dsmem(smraw, (unsigned)gl) : 0u;
    const unsigned off_cf = (unsigned)__cvta_generic_to_shared(cf) - sm_base + 4u * (unsigned)nt;
    const unsigned off_wsc = (unsigned)__cvta_generic_to_shared(wsc) - sm_base;
    const unsigned off_wt = (unsigned)__cvta_generic_to_shared(wt) - sm_base;
    const unsigned gmask = LPS == 32 ? 0xffffffffu : (((1u << LPS) - 1u) << (grp * LPS));
    // the group's own sample w, lane gl holding entries gl + LPS h (scores x[h], templates r[h]):
    // the maximum of the list -- largest Cf, then the lower template -- pushed into every CTA.
    // Cf bits + 1 order the valid entries above every padding entry (0); the group maximum is
    // taken on those 32 bits, and only when several lanes share it does a second reduction pick
    // the lowest template among them.
    // hn: the entry slots in use (warp-uniform; the second slot of widened lists is all padding at
    // most samples, and then skipped)
    auto finish_push = [&](int w, const float (&x)[EPL], const int (&r)[EPL], bool valid, int hn) {
        unsigned u = 0u, rr = 0xffffffffu;
        float xb = 0.f;
#pragma unroll
        for (int h = 0; h < EPL; ++h) {
            const int e = gl + LPS * h;
            if (h < hn && valid && e < keep && r[h] != kListPad) {
                const float q = fmaxf(x[h], 0.f);
                const unsigned uh = __float_as_uint(q * q * s_inm[r[h]]) + 1u;
                if (uh > u || (uh == u && (unsigned)r[h] < rr)) {
                    u = uh;
                    rr = (unsigned)r[h];
                    xb = x[h];
                }
            }
        }
        unsigned m = u;
#pragma unroll
        for (int o = LPS / 2; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        const unsigned cand = __ballot_sync(0xffffffffu, u == m) & gmask;
        unsigned rmin = rr;
        if (__any_sync(0xffffffffu, __popc(cand) > 1)) {
            rmin = u == m ? rr : 0xffffffffu;
#pragma unroll
            for (int o = LPS / 2; o > 0; o >>= 1) rmin = min(rmin, __shfl_xor_sync(0xffffffffu, rmin, o));
        }
        const int win = __ffs(__ballot_sync(0xffffffffu, u == m && (__popc(cand) == 1 || rr == rmin)) & gmask) - 1;
        const float xw = __shfl_sync(0xffffffffu, xb, win);
        const unsigned tw = __shfl_sync(0xffffffffu, rr, win);
        if (valid && gl < G) {
            const bool inner = w >= nt && w < W - nt;
            const float v = inner && m > 0u ? __uint_as_float(m - 1u) : 0.f;
            asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(rem + off_cf + 4u * (unsigned)w), "f"(v) : "memory");
            asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(rem + off_wsc + 4u * (unsigned)w), "f"(xw) : "memory");
            asm volatile("st.shared::cluster.s32 [%0], %1;" ::"r"(rem + off_wt + 4u * (unsigned)w), "r"((int)tw)
                         : "memory");
        }
    };
    for (int j0 = warp * kGroups; j0 < span; j0 += kWarps * kGroups) {
        const int j = j0 + grp;
        const bool valid = j < own;
        const int w = rank + G * j;
        int r[EPL];
        float x[EPL];
#pragma unroll
        for (int h = 0; h < EPL; ++h) {
            const int e = gl + LPS * h;
            const bool in = valid && e < keep && (h == 0 || s_wide[j]);
            r[h] = !in ? (int)kListPad : h == 0 ? RK[(size_t)j * ks + e] : rk_g[(size_t)w * KP + e];
            x[h] = !in ? 0.f : h == 0 ? SC[(size_t)j * ks + e] : sc_g[(size_t)w * KP + e];
        }
        finish_push(w, x, r, valid, EPL);
    }
    cluster_sync_all<G>();

    int n_total = 0, iters = 0;
    int* sp_w = out.sp_w + (int64_t)b * out.cap;
    int* sp_t = out.sp_t + (int64_t)b * out.cap;
    float* sp_amp = out.sp_amp + (int64_t)b * out.cap;
    int* sp_iter = out.sp_iter + (int64_t)b * out.cap;
    for (int it = 0; it < max_iters; ++it) {
        // ---- B1: the max pool of the replicated maxima (block prefix / suffix maxima), acceptance
        for (int blk = warp; blk * L2 < n; blk += kWarps) {
            const int b0 = blk * L2, b1 = min(n, b0 + L2);
            float carry = -FLT_MAX;
            for (int c0 = b0; c0 < b1; c0 += 32) {
                const int i = c0 + lane;
                float v = i < b1 ? cf[i] : -FLT_MAX;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const float o = __shfl_up_sync(0xffffffffu, v, d);
                    if (lane >= d) v = fmaxf(v, o);
                }
                v = fmaxf(v, carry);
                if (i < b1) pg[i] = v;
                carry = __shfl_sync(0xffffffffu, v, 31);
            }
            carry = -FLT_MAX;
            for (int c1 = b1; c1 > b0; c1 -= 32) {
                const int i = c1 - 32 + lane;
                float v = i >= b0 ? cf[i] : -FLT_MAX;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const float o = __shfl_down_sync(0xffffffffu, v, d);
                    if (lane + d < 32) v = fmaxf(v, o);
                }
                v = fmaxf(v, carry);
                if (i >= b0) ph[i] = v;
                carry = __shfl_sync(0xffffffffu, v, 0);
            }
        }
        __syncthreads();
        for (int w = tid; w < W; w += NTHR) {
            const float c = cf[w + nt];
            if (c > th2 && c == fmaxf(ph[w], pg[w + 2 * nt])) {
                const int tt = wt[w];
                const int q = atomicAdd(&s_cnt, 1);
                if (q < cap_it) {
                    s_aw[q] = w;
                    s_at[q] = tt;
                    s_aa[q] = wsc[w] / s_nm[tt];
                } else {
                    s_over = 1;
                }
            }
        }
        __syncthreads();
        // no CTA pushes the maxima phase C changes before every CTA has read this iteration's
        // replicas (max pool, acceptance): otherwise a CTA that runs behind could see some of them
        // lowered, accept other spikes and end the loop apart from the others.  The barrier's
        // arrival is here, its wait before C, with the ranking and the item table in between.
        cluster_arrive();
        const int total = min(s_cnt, cap_it);
        if (total == 0) {
            cluster_wait();
            break;
        }
        ++iters;
        // ---- B2: rank by sample; the own samples each spike's items cover ----
        for (int k = tid; k < total; k += NTHR) {
            const int w = s_aw[k];
            int r = 0;
            for (int q = 0; q < total; ++q) r += s_aw[q] < w;
            s_sw[r] = w;
            s_st[r] = s_at[k];
            s_sa[r] = s_aa[k];
            s_cb[r] = (s_at[k] * L2 + nt - w) * T;   // ctcP[t_k][w' - w + nt][t] at s_cb + w' T + t
            const int o = n_total + r;
            if (rank == 0 && o < out.cap) {
                sp_w[o] = w;
                sp_t[o] = s_at[k];
                sp_amp[o] = s_aa[k];
                sp_iter[o] = it;
            }
        }
        __syncthreads();
        if (warp == 0) {
            // spike k takes the samples [lo, hi) near it that no earlier spike took; its own ones
            // are lo' = the first w >= lo with w = rank (mod G), then every G-th
            int carry = 0;
            for (int k0 = 0; k0 < total; k0 += 32) {
                const int k = k0 + lane;
                int cnt = 0, first = 0;
                if (k < total) {
                    const int sw = s_sw[k];
                    const int lo = max(max(sw - nt, 0), k > 0 ? s_sw[k - 1] + nt + 1 : 0);
                    const int hi = min(W, sw + nt + 1);
                    first = lo + (((rank - lo) % G) + G) % G;
                    cnt = first < hi ? (hi - 1 - first) / G + 1 : 0;
                }
                int inc = cnt;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const int o = __shfl_up_sync(0xffffffffu, inc, d);
                    if (lane >= d) inc += o;
                }
                if (k < total) {
                    s_lo[k] = first;
                    s_pre[k] = carry + inc - cnt;
                }
                carry += __shfl_sync(0xffffffffu, inc, 31);
            }
            if (lane == 0) {
                s_pre[total] = carry;
                s_cnt = 0;   // read again only after the barrier ending C
            }
        }
        __syncthreads();
        // the item table: item q = own sample s_lo[k] + G (q - s_pre[k]) of the spike k whose
        // items hold q (32 threads per spike)
        for (int idx = tid; idx < total * 32; idx += NTHR) {
            const int k = idx >> 5;
            for (int q = s_pre[k] + (idx & 31); q < s_pre[k + 1]; q += 32) {
                s_itw[q] = s_lo[k] + G * (q - s_pre[k]);
                s_itk[q] = k;
            }
        }
        __syncthreads();
        cluster_wait();   // every CTA has read its replicas: pushes may start
        // ---- C: subtract the spikes from the listed scores of the own samples near them ----
        const int n_items = s_pre[total];
        constexpr int kPerWarp = kItems * kGroups;
        for (int q0 = warp * kPerWarp; q0 < n_items; q0 += kWarps * kPerWarp) {
            int wv[kItems], kv[kItems], jv[kItems], rv[kItems][EPL], hn[kItems];
            float xv[kItems][EPL], cv[kItems][EPL], cv2[kItems][EPL];
            bool two[kItems];
#pragma unroll
            for (int u = 0; u < kItems; ++u) {
                const int q = q0 + u * kGroups + grp;
                int w = -1, k = 0;
                if (q < n_items) {
                    w = s_itw[q];
                    k = s_itk[q];
                }
                wv[u] = w;
                kv[u] = k;
                jv[u] = w >= 0 ? (w - rank) / G : 0;
                two[u] = w >= 0 && k + 1 < total && s_sw[k + 1] - nt <= w;
                const bool wide = w >= 0 && s_wide[jv[u]];
#pragma unroll
                for (int h = 0; h < EPL; ++h) {
                    const int e = gl + LPS * h;
                    rv[u][h] = kListPad;
                    xv[u][h] = 0.f;
                    if (w >= 0 && e < keep && (h == 0 || wide)) {
                        rv[u][h] = h == 0 ? RK[(size_t)jv[u] * ks + e] : rk_g[(size_t)w * KP + e];
                        xv[u][h] = h == 0 ? SC[(size_t)jv[u] * ks + e] : sc_g[(size_t)w * KP + e];
                    }
                }
                // the slots any lane of the warp uses for this item
                hn[u] = EPL > 1 && __any_sync(0xffffffffu, wide) ? EPL : 1;
            }
#pragma unroll
            for (int u = 0; u < kItems; ++u) {
#pragma unroll
                for (int h = 0; h < EPL; ++h) {
                    cv[u][h] = cv2[u][h] = 0.f;
                    if (h < hn[u] && wv[u] >= 0 && gl + LPS * h < keep && rv[u][h] != kListPad) {
                        const int k = kv[u];
                        const int wo = wv[u] * T + rv[u][h];
                        cv[u][h] = __ldg(ctcP + (s_cb[k] + wo));
                        if (two[u]) cv2[u][h] = __ldg(ctcP + (s_cb[k + 1] + wo));
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < kItems; ++u) {
                const int w = wv[u];
                if (!__any_sync(0xffffffffu, w >= 0)) continue;
                float x[EPL];
#pragma unroll
                for (int h = 0; h < EPL; ++h) {
                    x[h] = 0.f;
                    const int e = gl + LPS * h;
                    if (h < hn[u] && w >= 0) {
                        const int k = kv[u];
                        float xe = fmaf(-s_sa[k], cv[u][h], xv[u][h]);
                        if (two[u]) {
                            xe = fmaf(-s_sa[k + 1], cv2[u][h], xe);
                            for (int kk = k + 2; kk < total && s_sw[kk] - nt <= w; ++kk) {   // rare: a third
                                const float c = e < keep && rv[u][h] != kListPad
                                                    ? __ldg(ctcP + (s_cb[kk] + w * T + rv[u][h]))
                                                    : 0.f;
                                xe = fmaf(-s_sa[kk], c, xe);
                            }
                        }
                        if (e < keep && rv[u][h] != kListPad) {
                            if (h == 0) SC[(size_t)jv[u] * ks + e] = xe;
                            else sc_g[(size_t)w * KP + e] = xe;
                        }
                        x[h] = xe;
                    }
                }
                finish_push(w, x, rv[u], w >= 0, hn[u]);
            }
        }
        n_total += total;
        cluster_sync_all<G>();   // every CTA holds every updated maximum before the next B1
    }
    if (rank == 0 && tid == 0) {
        out.n_spikes[b] = n_total;
        out.n_iters[b] = iters;
        if (n_total > out.cap || s_over) atomicOr(out.status + b, 1);
    }
}

// the opt-in shared memory per block, queried once (a function-local static: initialised once even
// when several host threads drive handles at the same time)
static int prune_smem_max() {
    static const int v = [] {
        int dev = 0, r = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&r, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
            cudaGetLastError();
            r = 0;
        }
        return r;
    }();
    return v;
}

// where the per-sample state of a window goes: bit 0 = maxima and slots in shared memory, bit 1 =
// the listed templates too, bit 2 = their scores too; -1 = the fixed part alone does not fit
int prune_mode(int W, int T, int nt, int keep) {
    const size_t lim = (size_t)prune_smem_max();
    const size_t f = prune_smem_fixed(W, T, nt) + 1024;
    if (f > lim) return -1;
    const size_t c = prune_smem_cf(W, nt);
    if (f + c > lim) return 0;
    const int ks = prune_stride(keep);
    const size_t r = prune_smem_ranks(W, ks);
    if (f + c + r > lim) return 1;
    return f + c + r + prune_smem_scores(W, ks) <= lim ? 7 : 3;
}

static size_t prune_smem(int W, int T, int nt, int keep, int mode) {
    const int ks = prune_stride(keep);
    return prune_smem_fixed(W, T, nt) + ((mode & 1) ? prune_smem_cf(W, nt) : 0) +
           ((mode & 2) ? prune_smem_ranks(W, ks) : 0) + ((mode & 4) ? prune_smem_scores(W, ks) : 0);
}

template <int LPS>
static cudaError_t launch_pruned_lps(const uint16_t* lrk, float* lsc, int keep, const float* ctcP, const float* nm,
                                     float th2, int W, int T, int nt, int max_iters, int nb, int mode, float* cf_scratch,
                                     unsigned char* slot_scratch, const MatchOut& out, cudaStream_t s) {
    const size_t smem = prune_smem(W, T, nt, keep, mode);
    auto kern = match_pruned_kernel<kPruneThreads, LPS>;
    cudaError_t e = raise_smem_limit((const void*)kern, smem);
    if (e != cudaSuccess) return e;
    kern<<<nb, kPruneThreads, smem, s>>>(lrk, lsc, keep, ctcP, nm, th2, W, T, nt, max_iters, mode, cf_scratch,
                                         slot_scratch, out);
    return cudaGetLastError();
}

template <int G, int NTHR, int LPS, int EPL>
static cudaError_t launch_pruned_cluster(const uint16_t* lrk, float* lsc, int keep, const float* ctcP,
                                         const float* nm, float th2, int W, int T, int nt, int max_iters, int nb,
                                         const MatchOut& out, cudaStream_t s) {
    const size_t smem = prune_cl_smem(W, T, nt, keep, G);
    auto kern = match_pruned_cluster_kernel<G, NTHR, LPS, EPL>;
    cudaError_t e = raise_smem_limit((const void*)kern, smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(nb * G));
    cfg.blockDim = dim3(NTHR);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = G;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, lrk, lsc, keep, ctcP, nm, th2, W, T, nt, max_iters, out);
}

// the cluster form when a CTA's share fits in shared memory: 4 CTAs of 512 threads per window for
// groups (one wave for 64 windows at up to 24 listed templates), 8 CTAs for a few windows
// (latency); lane groups of 16, one list entry per lane up to 16 entries, two up to 32
static cudaError_t try_pruned_cluster(const uint16_t* lrk, float* lsc, int keep, const float* ctcP,
                                      const float* nm, float th2, int W, int T, int nt, int max_iters, int nb,
                                      const MatchOut& out, cudaStream_t s, bool* done) {
    *done = false;
    const int G = nb <= 8 ? 8 : 4;
    if (W < 2 * G * nt || prune_cl_smem(W, T, nt, keep, G) + 1024 > (size_t)prune_smem_max()) return cudaSuccess;
    *done = true;
#define LSS_PCL(GG, EE) \
    launch_pruned_cluster<GG, 512, 16, EE>(lrk, lsc, keep, ctcP, nm, th2, W, T, nt, max_iters, nb, out, s)
    if (keep <= 16) return G == 8 ? LSS_PCL(8, 1) : LSS_PCL(4, 1);
    return G == 8 ? LSS_PCL(8, 2) : LSS_PCL(4, 2);
#undef LSS_PCL
}

cudaError_t launch_match_pruned(const uint16_t* lrk, float* lsc, int keep, const float* ctcP, const float* nm,
                                float th2, int W, int T, int nt, int max_iters, int nb, float* cf_scratch,
                                unsigned char* slot_scratch, const MatchOut& out, cudaStream_t s) {
    if (keep < 1 || keep > KP || keep > T || T > 1024) return cudaErrorInvalidValue;
    {
        bool done = false;
        const cudaError_t e = try_pruned_cluster(lrk, lsc, keep, ctcP, nm, th2, W, T, nt, max_iters, nb, out, s, &done);
        if (done || e != cudaSuccess) return e == cudaSuccess ? cudaGetLastError() : e;
    }
    const int mode = prune_mode(W, T, nt, keep);
    if (mode < 0 || (!(mode & 1) && (!cf_scratch || !slot_scratch))) return cudaErrorInvalidValue;
    if (keep <= 8)
        return launch_pruned_lps<8>(lrk, lsc, keep, ctcP, nm, th2, W, T, nt, max_iters, nb, mode, cf_scratch,
                                    slot_scratch, out, s);
    if (keep <= 16)
        return launch_pruned_lps<16>(lrk, lsc, keep, ctcP, nm, th2, W, T, nt, max_iters, nb, mode, cf_scratch,
                                     slot_scratch, out, s);
    return launch_pruned_lps<32>(lrk, lsc, keep, ctcP, nm, th2, W, T, nt, max_iters, nb, mode, cf_scratch,
                                 slot_scratch, out, s);
}

}  // namespace lss
