// kernels_match.cu -- the matching-pursuit loop of Kilosort template_matching.py:157-198 as one
// persistent kernel per batch: a thread-block cluster of G CTAs owns one window, each CTA a
// contiguous slice of its time samples.  Per iteration:
//
//   A  per-sample max / argmax over templates of Cf = relu(B)^2 / nm (first and last nt
//      samples zeroed), only for samples whose scores changed in the previous iteration;
//   B1 (2nt+1) max pool of that per-sample max; accept a sample when the pooled value
//      exceeds Th^2 and equals the sample's own max; amplitude B[w][iY] / nm[iY];
//   B2 write the accepted spikes, ordered by (iteration, sample) like the reference;
//   C  subtract every accepted spike: B[w'][:] -= amp * ctc[:, iY, w'-w+nt] for |w'-w| <= nt
//      and Xres[w'][:] -= amp * waveform[iY][w'-w+nt/2] for |w'-w| <= nt/2 -- as a gather
//      per output sample (each CTA updates only its own samples, so no atomics and a fixed
//      summation order).
//
// Phases are separated by hardware cluster barriers (barrier.cluster arrive.release /
// wait.acquire); data shared between CTAs goes through L2 with .cg loads.  No spin-waits,
// no host round trips; the loop ends when an iteration accepts nothing (the same decision
// in every CTA) or after max_iters.
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

template <int G>
__global__ void __launch_bounds__(kMatchThreads)
match_kernel(float* __restrict__ Bt, float* __restrict__ Xres, const float* __restrict__ ctcP,
             const float* __restrict__ pre_wf, const float* __restrict__ nm, float th2, int W, int T, int C,
             int nt, int max_iters, MatchScratch sc, MatchOut out) {
    extern __shared__ float smem[];
    const int b = blockIdx.x / G;
    const int rank = (G == 1) ? 0 : (int)cluster_rank();
    const int span = (W + G - 1) / G;
    const int lo = min(W, rank * span), hi = min(W, lo + span);
    const int halo = hi - lo + 2 * nt;
    float* s_cf = smem;                                   // [halo]
    int* s_t = reinterpret_cast<int*>(s_cf + halo);      // [halo]
    float* s_amp = reinterpret_cast<float*>(s_t + halo); // [halo]
    __shared__ int s_cnt[G];
    __shared__ int s_red[kMatchThreads / 32];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = kMatchThreads / 32;
    const int L2 = 2 * nt + 1, hw = nt / 2;
    float* B = Bt + (int64_t)b * W * T;
    float* X = Xres + (int64_t)b * W * C;
    float* cfmax = sc.cfmax + (int64_t)b * W;
    int* imax = sc.imax + (int64_t)b * W;
    int* at_t = sc.at_t + (int64_t)b * W;
    float* at_amp = sc.at_amp + (int64_t)b * W;
    unsigned char* dirty = sc.dirty + (int64_t)b * W;
    int* cta_cnt = sc.cta_cnt + (int64_t)b * 2 * G;
    int* sp_w = out.sp_w + (int64_t)b * out.cap;
    int* sp_t = out.sp_t + (int64_t)b * out.cap;
    float* sp_amp = out.sp_amp + (int64_t)b * out.cap;
    int* sp_iter = out.sp_iter + (int64_t)b * out.cap;

    if (G > 1 && rank != (unsigned)(blockIdx.x % G) && tid == 0) atomicOr(out.status + b, 2);
    for (int w = lo + tid; w < hi; w += kMatchThreads) dirty[w] = 1;
    __syncthreads();

    int n_total = 0, iters = 0;
    for (int it = 0; it < max_iters; ++it) {
        // ---- A: per-sample max / argmax over templates (changed samples only) ----
        for (int w = lo + warp; w < hi; w += nwarps) {
            if (!dirty[w]) continue;
            float best = 0.f;
            int bi = 0;
            if (w >= nt && w < W - nt) {
                best = -1.f;
                bi = 0x7fffffff;
                const float* row = B + (int64_t)w * T;
                for (int t = lane; t < T; t += 32) {
                    const float r = fmaxf(row[t], 0.f);
                    const float v = r * r / nm[t];
                    if (v > best) { best = v; bi = t; }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const float ob = __shfl_xor_sync(0xffffffffu, best, o);
                    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                    if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
                }
            }
            if (lane == 0) { cfmax[w] = best; imax[w] = bi; }
        }
        group_barrier<G>();

        // ---- B1: pooled max and acceptance on the own slice ----
        for (int i = tid; i < halo; i += kMatchThreads) {
            const int w = lo - nt + i;
            s_cf[i] = (w >= 0 && w < W) ? __ldcg(cfmax + w) : -FLT_MAX;
        }
        __syncthreads();
        int my_cnt = 0;
        for (int w = lo + tid; w < hi; w += kMatchThreads) {
            const int i = w - lo + nt;
            float cm = -FLT_MAX;
            for (int d = -nt; d <= nt; ++d) cm = fmaxf(cm, s_cf[i + d]);
            const float cf = s_cf[i];
            int tt = -1;
            float amp = 0.f;
            if (cm > th2 && cf == cm) {
                tt = imax[w];
                amp = B[(int64_t)w * T + tt] / nm[tt];
                ++my_cnt;
            }
            at_t[w] = tt;
            at_amp[w] = amp;
        }
        my_cnt = __reduce_add_sync(0xffffffffu, my_cnt);
        if (lane == 0) s_red[warp] = my_cnt;
        __syncthreads();
        if (tid == 0) {
            int c = 0;
            for (int i = 0; i < nwarps; ++i) c += s_red[i];
            cta_cnt[(it & 1) * G + rank] = c;
        }
        group_barrier<G>();

        // ---- totals: the same numbers in every CTA of the cluster ----
        if (tid < G) s_cnt[tid] = __ldcg(cta_cnt + (it & 1) * G + tid);
        __syncthreads();
        int total = 0, base = n_total;
        for (int r = 0; r < G; ++r) {
            total += s_cnt[r];
            if (r < rank) base += s_cnt[r];
        }
        if (total == 0) break;
        ++iters;

        // ---- B2: record the own slice's spikes in sample order ----
        if (warp == 0) {
            int run = base;
            for (int w0 = lo; w0 < hi; w0 += 32) {
                const int w = w0 + lane;
                const int tt = (w < hi) ? at_t[w] : -1;
                const unsigned m = __ballot_sync(0xffffffffu, tt >= 0);
                if (tt >= 0) {
                    const int slot = run + __popc(m & ((1u << lane) - 1u));
                    if (slot < out.cap) {
                        sp_w[slot] = w;
                        sp_t[slot] = tt;
                        sp_amp[slot] = at_amp[w];
                        sp_iter[slot] = it;
                    }
                }
                run += __popc(m);
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
        for (int wp = lo + warp; wp < hi; wp += nwarps) {
            const int i0 = wp - lo;   // s_t[i0 + e] is the sample wp - nt + e
            bool any = false;
            for (int e0 = 0; e0 < L2; e0 += 32) {
                const int e = e0 + lane;
                unsigned m = __ballot_sync(0xffffffffu, e < L2 && s_t[i0 + e] >= 0);
                while (m) {
                    const int ee = e0 + __ffs(m) - 1;
                    m &= m - 1;
                    any = true;
                    const int ts = s_t[i0 + ee];
                    const float a = s_amp[i0 + ee];
                    const int l = 2 * nt - ee;               // = wp - w + nt
                    const float* crow = ctcP + ((int64_t)ts * L2 + l) * T;
                    float* brow = B + (int64_t)wp * T;
                    for (int t = lane; t < T; t += 32) brow[t] = fmaf(-a, __ldg(crow + t), brow[t]);
                    const int dw = nt - ee;                   // = wp - w
                    if (dw >= -hw && dw <= hw) {
                        const float* wrow = pre_wf + ((int64_t)ts * nt + (dw + hw)) * C;
                        float* xrow = X + (int64_t)wp * C;
                        for (int c = lane; c < C; c += 32) xrow[c] = fmaf(-a, __ldg(wrow + c), xrow[c]);
                    }
                }
            }
            if (lane == 0) dirty[wp] = any ? 1 : 0;
        }
        n_total += total;
        __syncthreads();
    }
    if (rank == 0 && tid == 0) {
        out.n_spikes[b] = n_total;
        out.n_iters[b] = iters;
        if (n_total > out.cap) atomicOr(out.status + b, 1);
    }
}

cudaError_t launch_match(float* Bt, float* Xres, const float* ctcP, const float* pre_wf, const float* nm, float th2,
                         int W, int T, int C, int nt, int max_iters, int nb, const MatchScratch& sc,
                         const MatchOut& out, cudaStream_t s) {
    constexpr int G = kMatchCluster;
    const int span = (W + G - 1) / G;
    const size_t smem = (size_t)(span + 2 * nt) * 12;
    auto kern = match_kernel<G>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nb * G, 1, 1);
    cfg.blockDim = dim3(kMatchThreads, 1, 1);
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

}  // namespace lss
