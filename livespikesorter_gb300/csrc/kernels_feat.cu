// kernels_feat.cu -- per-spike PC features, position and final-cluster assignment.
//
//   tF[n][k] = sum_r Xres[w + r - nt/2][iCC[n][iU[t]]] * wPCA[k][r] + amp * Ucc[n][t][k]
//              (Kilosort template_matching.py:50-51)
//   (x, y)   = sum_n (mass_n / sum mass) * (xc, yc)[iCC[n][iU[t]]],  mass_n = sum_k tF[n][k]^2
//              (Kilosort postprocessing.py:33-46)
//   cluster  = nearest final-cluster centroid in (x, y), first on ties
//              (OnlineSpikesV2::closestCluster, OnlineSpikesV2.cu:1058-1074); or, with the PC-score
//              rule, argmax_k 2 tF.mu_k - |mu_k|^2 over the clusters whose centroid lies within R
//              of (x, y) (first on ties), -1 when none does (OnlineKilosort.py:233-284)
//
// One warp per spike; records are written straight into host-mapped memory.
#include "lss_kernels.cuh"

#include <algorithm>
#include <cfloat>

namespace lss {

__global__ void rec_offsets_kernel(const int* __restrict__ n_spikes, int nb, int cap, int* __restrict__ off) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int acc = 0;
    for (int b = 0; b < nb; ++b) {
        off[b] = acc;
        acc += min(n_spikes[b], cap);
    }
    off[nb] = acc;
}

void launch_rec_offsets(const MatchOut& out, int nb, int* rec_offset, cudaStream_t s) {
    rec_offsets_kernel<<<1, 32, 0, s>>>(out.n_spikes, nb, out.cap, rec_offset);
}

constexpr int kFeatWarps = 8;
constexpr int kFeatMaxK = 8;   // PCs (the loader refuses more)

// The tail of a spike record from its features sf[0 .. nC K) (in shared memory, the warp's own):
// mass per nearest channel, the weighted position, the cluster, and the record itself.
__device__ __forceinline__ void finish_record(const float* sf, int lane, int b, int w, int t, int iter, float amp,
                                              int64_t peak, int C, int K, int nC, const int64_t* __restrict__ iCC,
                                              const float* __restrict__ xc, const float* __restrict__ yc,
                                              const float* __restrict__ centroids, int n_final,
                                              const float* __restrict__ cpca, const float* __restrict__ cpca_nm,
                                              float r2, SpikeRec* __restrict__ rec, int batch_base) {
    const int nf = nC * K;
    // mass per nearest channel, then the weighted position
    __syncwarp();
    float mx = 0.f, my = 0.f, ms = 0.f;
    if (lane < nC) {
        float mass = 0.f;
        for (int k = 0; k < K; ++k) mass = fmaf(sf[lane * K + k], sf[lane * K + k], mass);
        const int64_t ch = iCC[(int64_t)lane * C + peak];
        mx = xc[ch] * mass;
        my = yc[ch] * mass;
        ms = mass;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx += __shfl_xor_sync(0xffffffffu, mx, o);
        my += __shfl_xor_sync(0xffffffffu, my, o);
        ms += __shfl_xor_sync(0xffffffffu, ms, o);
    }
    const float x = mx / ms, y = my / ms;
    int bi = 0x7fffffff;
    if (cpca) {
        // PC score among the clusters within R: squares and sums rounded separately, as
        // elementwise float32 tensor arithmetic does (no fused multiply-add on the distance)
        float bs = -FLT_MAX;
        bool any = false;
        for (int j = lane; j < n_final; j += 32) {
            const float dx = __fsub_rn(x, centroids[2 * j]), dy = __fsub_rn(y, centroids[2 * j + 1]);
            if (!(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) <= r2)) continue;
            any = true;
            const float* mu = cpca + (int64_t)j * nf;
            float dot = 0.f;
            for (int p = 0; p < nf; ++p) dot = fmaf(sf[p], mu[p], dot);
            const float sc = __fsub_rn(__fmul_rn(2.f, dot), cpca_nm[j]);
            if (sc > bs || bi == 0x7fffffff) { bs = sc; bi = j; }
        }
        any = __any_sync(0xffffffffu, any);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float os = __shfl_xor_sync(0xffffffffu, bs, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (oi != 0x7fffffff && (bi == 0x7fffffff || os > bs || (os == bs && oi < bi))) { bs = os; bi = oi; }
        }
        if (!any) bi = -1;
    } else {
        // nearest centroid
        float bd = FLT_MAX;
        for (int j = lane; j < n_final; j += 32) {
            const float dx = x - centroids[2 * j], dy = y - centroids[2 * j + 1];
            const float d = dx * dx + dy * dy;
            if (d < bd) { bd = d; bi = j; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float od = __shfl_xor_sync(0xffffffffu, bd, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (od < bd || (od == bd && oi < bi)) { bd = od; bi = oi; }
        }
        if (bi == 0x7fffffff) bi = 0;   // NaN position (zero feature energy): first cluster
    }
    // the 288-byte record as 18 16-byte stores (it goes to host-mapped memory, where every store
    // is a transaction of its own): lanes 0 and 1 the header, lanes 2 .. 17 the 64 features
    static_assert(sizeof(SpikeRec) == 18 * 16, "SpikeRec is 18 16-byte words");
    uint4 v;
    if (lane == 0) {
        v = make_uint4((uint32_t)(batch_base + b), (uint32_t)w, (uint32_t)t, (uint32_t)iter);
    } else if (lane == 1) {
        v = make_uint4(__float_as_uint(amp), __float_as_uint(x), __float_as_uint(y), (uint32_t)bi);
    } else if (lane < 18) {
        const float* f = sf + 4 * (lane - 2);
        v = make_uint4(__float_as_uint(f[0]), __float_as_uint(f[1]), __float_as_uint(f[2]), __float_as_uint(f[3]));
    }
    if (lane < 18) reinterpret_cast<uint4*>(rec)[lane] = v;
}


__global__ void __launch_bounds__(kFeatWarps * 32)
features_kernel(const float* __restrict__ Xres, MatchOut out, int nb, int W, int C, int T, int K, int nt, int nC,
                const float* __restrict__ wPCA, const int64_t* __restrict__ iCC, const int64_t* __restrict__ iU,
                const float* __restrict__ Ucc, const float* __restrict__ xc, const float* __restrict__ yc,
                const float* __restrict__ centroids, int n_final, const float* __restrict__ cpca,
                const float* __restrict__ cpca_nm, float r2, const int* __restrict__ rec_offset,
                SpikeRec* __restrict__ recs, int batch_base) {
    const int lane = threadIdx.x & 31;
    const int total = rec_offset[nb];
    __shared__ float s_f[kFeatWarps][64];
    float* sf = s_f[threadIdx.x >> 5];
    for (int gw = blockIdx.x * kFeatWarps + (threadIdx.x >> 5); gw < total; gw += gridDim.x * kFeatWarps) {
    // locate the batch of record gw (nb is small: linear search)
    int b = 0;
    while (b + 1 < nb && rec_offset[b + 1] <= gw) ++b;
    const int slot = gw - rec_offset[b];
    const int64_t so = (int64_t)b * out.cap + slot;
    const int w = out.sp_w[so], t = out.sp_t[so], iter = out.sp_iter[so];
    const float amp = out.sp_amp[so];
    const float* X = Xres + (int64_t)b * W * C;
    const int hw = nt / 2;
    const int64_t peak = iU[t];

    // lpc lanes per nearest channel, each over a contiguous run of the nt taps for all K components
    // (every residual sample loaded once); the channel's first lane adds the others' partial sums
    // in lane order, then the amplitude term
    __syncwarp();
    sf[lane] = 0.f;
    sf[lane + 32] = 0.f;
    __syncwarp();
    const int lpc = nC >= 32 ? 1 : 32 / nC;
    const int part = lane % lpc, chunk = (nt + lpc - 1) / lpc;
    const int r0 = part * chunk, r1 = min(nt, r0 + chunk);
    for (int n0 = 0; n0 < nC; n0 += 32 / lpc) {
        const int n = n0 + lane / lpc;
        const bool have = lane / lpc < 32 / lpc && n < nC;
        float acc[kFeatMaxK];
#pragma unroll
        for (int k = 0; k < kFeatMaxK; ++k) acc[k] = 0.f;
        if (have) {
            const float* xc_ = X + (int64_t)(w - hw) * C + iCC[(int64_t)n * C + peak];
            for (int r = r0; r < r1; ++r) {
                const float x = xc_[(int64_t)r * C];
#pragma unroll
                for (int k = 0; k < kFeatMaxK; ++k)
                    if (k < K) acc[k] = fmaf(x, wPCA[k * nt + r], acc[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < kFeatMaxK; ++k) {
            float tot = acc[k];
            for (int q = 1; q < lpc; ++q) tot += __shfl_sync(0xffffffffu, acc[k], (lane + q) & 31);
            if (have && part == 0 && k < K) sf[n * K + k] = tot + amp * Ucc[((int64_t)n * T + t) * K + k];
        }
    }
    finish_record(sf, lane, b, w, t, iter, amp, peak, C, K, nC, iCC, xc, yc, centroids, n_final, cpca, cpca_nm, r2,
                  recs + gw, batch_base);
    }
}

void launch_features(const float* Xres, const MatchOut& out, int nb, int W, int C, int T, int K, int nt, int nC,
                     const float* wPCA, const int64_t* iCC, const int64_t* iU, const float* Ucc, const float* xc,
                     const float* yc, const float* centroids, int n_final, const float* cpca, const float* cpca_nm,
                     float r2, const int* rec_offset, SpikeRec* recs, int batch_base, cudaStream_t s) {
    const int max_recs = nb * out.cap;
    const int blocks = std::min((max_recs + kFeatWarps - 1) / kFeatWarps, 2048);
    features_kernel<<<blocks, kFeatWarps * 32, 0, s>>>(Xres, out, nb, W, C, T, K, nt, nC, wPCA, iCC, iU, Ucc, xc,
                                                       yc, centroids, n_final, cpca, cpca_nm, r2, rec_offset, recs,
                                                       batch_base);
}

// ---------------------------------------------------------------------------------------------
// The same records without the residual.  The features are the basis projection of the final
// residual, and the residual is the whitened window minus the accepted spikes' waveforms
// wf[t'][r][c] = sum_k' Wall3[t'][k'][c] wPCA[k'][r], so (both sums linear)
//   sum_r Xres[w + r - nt/2][c] wPCA[k][r]
//     = Bpc[w][k][c] - sum_{s': |w - w_s'| < nt} amp_s' sum_k' Wall3[t_s'][k'][c] P[k][k'][w - w_s']
// with Bpc the basis convolution the projection already used and P the basis cross-correlation
// P[k][k'][d] = sum_r wPCA[k][r] wPCA[k'][d + r] (0 <= r, d + r < nt).  A spike's features then
// cost nC K terms per overlapping spike instead of a pass over the whole residual, and the
// residual is never written.  (The reference subtracts the same waveforms from the residual in
// float32 and projects the result, template_matching.py:50-51 and :193-202; the two agree to
// float32 rounding.)
// FMT: 0 = Bpc in fp32; 1 = Bpc as an fp32 pair (hi + lo, the tf32 split); 2 = a BF16 pair.
// One warp per spike; lane n + nC j accumulates the overlapping spikes of slice j at nearest
// channel n, reading the channel-major template copy Wall3T[t][c][k] (K contiguous values).
// ---------------------------------------------------------------------------------------------
template <int FMT>
__device__ __forceinline__ float bpc_value(const void* hi, const void* lo, int64_t i) {
    if constexpr (FMT == 2) {
        return __uint_as_float((uint32_t)reinterpret_cast<const uint16_t*>(hi)[i] << 16) +
               __uint_as_float((uint32_t)reinterpret_cast<const uint16_t*>(lo)[i] << 16);
    } else if constexpr (FMT == 1) {
        return reinterpret_cast<const float*>(hi)[i] + reinterpret_cast<const float*>(lo)[i];
    } else {
        return reinterpret_cast<const float*>(hi)[i];
    }
}

constexpr int kNearCap = 64;   // overlapping spikes gathered per round (a multiple of 32 more than J - 1)

template <int FMT, int KC>
__global__ void __launch_bounds__(kFeatWarps * 32, 4)
features_direct_kernel(const void* __restrict__ bpc_hi, const void* __restrict__ bpc_lo, MatchOut out, int nb, int W,
                       int C, int T, int K, int nt, int nC, const float* __restrict__ wall3t,
                       const float* __restrict__ xcorr, const int64_t* __restrict__ iCC,
                       const int64_t* __restrict__ iU, const float* __restrict__ Ucc, const float* __restrict__ xc,
                       const float* __restrict__ yc, const float* __restrict__ centroids, int n_final,
                       const float* __restrict__ cpca, const float* __restrict__ cpca_nm, float r2,
                       const int* __restrict__ rec_offset, SpikeRec* __restrict__ recs, int batch_base) {
    // KC: the component count when known at compile time (0: K at run time, up to kFeatMaxK)
    constexpr int KM = KC > 0 ? KC : kFeatMaxK;
    if (KC > 0 && K != KC) return;
    extern __shared__ float s_p[];   // P[d + nt - 1][k][k'], (2 nt - 1) K K
    __shared__ float s_f[kFeatWarps][64];
    __shared__ int s_nd[kFeatWarps][kNearCap + 32], s_ntp[kFeatWarps][kNearCap + 32];
    __shared__ float s_na[kFeatWarps][kNearCap + 32];
    const int nd = 2 * nt - 1;
    for (int i = threadIdx.x; i < K * K * nd; i += blockDim.x) {
        const int d = i / (K * K), kk = i - d * K * K;      // xcorr is [k][k'][d]
        s_p[i] = xcorr[(int64_t)kk * nd + d];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int total = rec_offset[nb];
    float* sf = s_f[threadIdx.x >> 5];
    // lane = n + nC j: nearest channel n, neighbour slice j of J (every J-th overlapping spike)
    const int J = nC >= 32 ? 1 : 32 / nC;
    const int n = lane % nC, jj = lane / nC;
    const bool act = jj < J && n < nC;
    for (int gw = blockIdx.x * kFeatWarps + (threadIdx.x >> 5); gw < total; gw += gridDim.x * kFeatWarps) {
        int b = 0;
        while (b + 1 < nb && rec_offset[b + 1] <= gw) ++b;
        const int slot = gw - rec_offset[b];
        const int64_t so = (int64_t)b * out.cap + slot;
        const int w = out.sp_w[so], t = out.sp_t[so], iter = out.sp_iter[so];
        const float amp = out.sp_amp[so];
        const int64_t peak = iU[t];
        const int64_t ch = iCC[(int64_t)n * C + peak];
        float acc[KM];
#pragma unroll
        for (int k = 0; k < KM; ++k) acc[k] = 0.f;
        // every accepted spike of the batch whose waveform overlaps this spike's nt samples
        // (itself included), gathered in list order into the warp's table (kNearCap at a time);
        // slice j then takes the ones whose rank among them is j mod J, all slices at once
        const int n_sp = min(out.n_spikes[b], out.cap);
        const int* sw = out.sp_w + (int64_t)b * out.cap;
        const int* st = out.sp_t + (int64_t)b * out.cap;
        const float* sa = out.sp_amp + (int64_t)b * out.cap;
        int* nd = s_nd[threadIdx.x >> 5];
        int* ntp = s_ntp[threadIdx.x >> 5];
        float* na = s_na[threadIdx.x >> 5];
        const int kd = KC > 0 ? KC : K;
        auto apply = [&](int cnt) {
            // entries jj, jj + J, ... of the table, in order
            if (act) {
#pragma unroll 2
                for (int e = jj; e < cnt; e += J) {
                    const int dd = nd[e], t2 = ntp[e];
                    const float a2 = na[e];
                    const float* u = wall3t + ((int64_t)t2 * C + ch) * kd;
                    const float* pd = s_p + (dd + nt - 1) * kd * kd;
                    float uk[KM];
#pragma unroll
                    for (int k2 = 0; k2 < KM; ++k2) uk[k2] = (KC > 0 || k2 < K) ? __ldg(u + k2) : 0.f;
#pragma unroll
                    for (int k = 0; k < KM; ++k) {
                        if (KC == 0 && k >= K) break;
                        float sum = 0.f;
#pragma unroll
                        for (int k2 = 0; k2 < KM; ++k2)
                            if (KC > 0 || k2 < K) sum = fmaf(uk[k2], pd[k * kd + k2], sum);
                        acc[k] = fmaf(-a2, sum, acc[k]);
                    }
                }
            }
            __syncwarp();
        };
        // the table restarts at a multiple of J entries, so an entry's rank mod J is its slice
        int cnt = 0;
        for (int i0 = 0; i0 < n_sp; i0 += 32) {
            const int i = i0 + lane;
            const int d = i < n_sp ? w - sw[i] : nt;
            const bool near = d > -nt && d < nt;
            const unsigned m = __ballot_sync(0xffffffffu, near);
            if (cnt + __popc(m) > kNearCap) {
                const int full = cnt - cnt % J;   // apply whole rounds of J, keep the rest
                apply(full);
                const int rest = cnt - full;
                const int sd = lane < rest ? nd[full + lane] : 0, stt = lane < rest ? ntp[full + lane] : 0;
                const float sav = lane < rest ? na[full + lane] : 0.f;
                __syncwarp();
                if (lane < rest) {
                    nd[lane] = sd;
                    ntp[lane] = stt;
                    na[lane] = sav;
                }
                __syncwarp();
                cnt = rest;
            }
            if (near) {
                const int pos = cnt + __popc(m & ((1u << lane) - 1u));
                nd[pos] = d;
                ntp[pos] = st[i];
                na[pos] = sa[i];
            }
            __syncwarp();
            cnt += __popc(m);
        }
        apply(cnt);
        // slices summed in slice order into lane n, then the convolution and the amplitude term
#pragma unroll
        for (int k = 0; k < KM; ++k) {
            float tot = acc[k];
            for (int q = 1; q < J; ++q) tot += __shfl_sync(0xffffffffu, acc[k], (lane + q * nC) & 31);
            acc[k] = tot;
        }
        __syncwarp();
        sf[lane] = 0.f;
        sf[lane + 32] = 0.f;
        __syncwarp();
        if (act && jj == 0) {
#pragma unroll
            for (int k = 0; k < KM; ++k) {
                if (KC == 0 && k >= K) break;
                const float base = bpc_value<FMT>(bpc_hi, bpc_lo, (((int64_t)b * W + w) * K + k) * C + ch);
                sf[n * K + k] = (base + acc[k]) + amp * Ucc[((int64_t)n * T + t) * K + k];   // acc = -(overlaps)
            }
        }
        finish_record(sf, lane, b, w, t, iter, amp, peak, C, K, nC, iCC, xc, yc, centroids, n_final, cpca, cpca_nm,
                      r2, recs + gw, batch_base);
    }
}

void basis_xcorr(const float* wPCA, int K, int nt, float* P) {
    const int nd = 2 * nt - 1;
    for (int k = 0; k < K; ++k)
        for (int k2 = 0; k2 < K; ++k2)
            for (int d = -(nt - 1); d <= nt - 1; ++d) {
                double acc = 0.0;
                for (int r = 0; r < nt; ++r)
                    if (d + r >= 0 && d + r < nt) acc += (double)wPCA[(size_t)k * nt + r] * wPCA[(size_t)k2 * nt + d + r];
                P[((size_t)k * K + k2) * nd + d + nt - 1] = (float)acc;
            }
}

void launch_features_direct(const void* bpc_hi, const void* bpc_lo, int fmt, const MatchOut& out, int nb, int W,
                            int C, int T, int K, int nt, int nC, const float* wall3t, const float* xcorr,
                            const int64_t* iCC, const int64_t* iU, const float* Ucc, const float* xc, const float* yc,
                            const float* centroids, int n_final, const float* cpca, const float* cpca_nm, float r2,
                            const int* rec_offset, SpikeRec* recs, int batch_base, cudaStream_t s) {
    const int max_recs = nb * out.cap;
    const int blocks = std::min((max_recs + kFeatWarps - 1) / kFeatWarps, 2048);
    const size_t smem = sizeof(float) * (size_t)K * K * (2 * nt - 1);
    // six components (Kilosort's default basis) unrolled exactly, any other count up to 8 generic
    auto kern = K == 6 ? (fmt == 2 ? features_direct_kernel<2, 6>
                                   : (fmt == 1 ? features_direct_kernel<1, 6> : features_direct_kernel<0, 6>))
                       : (fmt == 2 ? features_direct_kernel<2, 0>
                                   : (fmt == 1 ? features_direct_kernel<1, 0> : features_direct_kernel<0, 0>));
    kern<<<blocks, kFeatWarps * 32, smem, s>>>(bpc_hi, bpc_lo, out, nb, W, C, T, K, nt, nC, wall3t, xcorr, iCC, iU, Ucc,
                                               xc, yc, centroids, n_final, cpca, cpca_nm, r2, rec_offset, recs,
                                               batch_base);
}

}  // namespace lss
