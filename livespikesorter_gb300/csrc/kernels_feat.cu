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
    const int nf = nC * K;

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
    SpikeRec* rec = recs + gw;
    rec->feat[lane] = sf[lane];
    rec->feat[lane + 32] = sf[lane + 32];
    if (lane == 0) {
        rec->batch = batch_base + b;
        rec->w = w;
        rec->t = t;
        rec->iter = iter;
        rec->amp = amp;
        rec->x = x;
        rec->y = y;
        rec->cluster = bi;
    }
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

}  // namespace lss
