// proposal.cu -- the learned proposal gate (include/lss_proposal.h): the network's kernels
// (forward, window loss, backward, Adam), the trainer handle, and the sorter-side gate that closes
// score cells before the matching loop.
//
// All kernels are plain FP32 SIMT: the network is small (65,153 parameters, 7-tap convolutions
// over 16 or 64 channels) and its tiles (128 samples x 64 output channels per block, staged input
// rows and weights in shared memory) keep every operand on chip for 16 input channels at a time.
// Reductions over examples are written as per-example partials and summed in example order, so a
// training step is deterministic.
#include "../../include/lss_proposal.h"
#include "oss_input.hpp"
#include "proposal.hpp"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

namespace lss {

extern thread_local std::string g_handleless_error;   // sorter.cu

namespace {

constexpr int kNbc = LSS_PROP_CHANNELS, kHid = LSS_PROP_HIDDEN, kTaps = LSS_PROP_TAPS, kPad = kTaps / 2;
constexpr int kWin = LSS_PROP_WINDOW;
constexpr int kTile = 128;                        // output samples per convolution block
constexpr int kCi = 16;                           // input channels staged per pass
constexpr int kXPitch = kTile + 2 * kPad + 1;     // 135 (odd): consecutive channel rows in different banks
constexpr size_t kGateBytes = size_t(256) << 20;  // activation buffer of one gate chunk

struct Layer {
    int out, in;
    size_t w, b;   // offsets in the flat parameter vector
};
constexpr Layer kLayers[4] = {{kHid, kNbc, 0, 7168}, {kHid, kHid, 7232, 35904}, {kHid, kHid, 35968, 64640},
                              {1, kHid, 64704, 65152}};
static_assert(kLayers[3].b + 1 == LSS_PROP_N_PARAMS, "parameter layout");

struct CudaFail {
    std::string msg;
};

#define PROP_CUDA(call)                                                                            \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) throw CudaFail{std::string(#call) + ": " + cudaGetErrorString(e_)}; \
    } while (0)

__device__ __forceinline__ float ld_w(const float* p) { return __ldg(p); }
__device__ __forceinline__ float ld_w(const __nv_bfloat16* p) { return __bfloat162float(*p); }

// x[e][i][l] = Z[pairs[e].x][l][pairs[e].y + i] (0 past the last channel): one neighbourhood of
// one whitened window, channel-major.  Block: 64 samples of one example.
__global__ void __launch_bounds__(256) gather_kernel(const float* __restrict__ Z, int W, int C,
                                                     const int2* __restrict__ pairs, float* __restrict__ x) {
    __shared__ float t[64][kNbc + 1];
    const int e = blockIdx.y, l0 = blockIdx.x * 64;
    const int2 pc = pairs[e];
    const float* zr = Z + (size_t)pc.x * W * C;
    for (int q = threadIdx.x; q < 64 * kNbc; q += blockDim.x) {
        const int ll = q / kNbc, i = q - ll * kNbc, l = l0 + ll, c = pc.y + i;
        t[ll][i] = (l < W && c < C) ? zr[(size_t)l * C + c] : 0.f;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < 64 * kNbc; q += blockDim.x) {
        const int i = q / 64, ll = q - i * 64, l = l0 + ll;
        if (l < W) x[((size_t)e * kNbc + i) * W + l] = t[ll][i];
    }
}

// out[e][o][l] = act(bias[o] + sum_i sum_k w[o][i][k] in[e][i][l + k - 3]) for 64 outputs, zeroed
// where mask[e][o][l] <= 0 (the ReLU of the layer below, in the data gradient).  Block: 128
// samples of one example; warp w owns outputs 8w..8w+7, lane j the samples j, j+32, j+64, j+96.
template <typename WT>
__global__ void __launch_bounds__(256) conv64_kernel(const float* __restrict__ in, int cin, int L,
                                                     const WT* __restrict__ w, const float* __restrict__ bias,
                                                     const float* __restrict__ mask, int relu,
                                                     float* __restrict__ out) {
    __shared__ float ws[kHid * kCi * kTaps];
    __shared__ float xs[kCi * kXPitch];
    const int e = blockIdx.y, l0 = blockIdx.x * kTile;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, o0 = warp * 8;
    float acc[8][4];
#pragma unroll
    for (int o = 0; o < 8; ++o)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[o][j] = 0.f;
    const float* inb = in + (size_t)e * cin * L;
    for (int c0 = 0; c0 < cin; c0 += kCi) {
        const int nci = min(kCi, cin - c0);
        __syncthreads();
        for (int q = threadIdx.x; q < kHid * kCi * kTaps; q += blockDim.x) {
            const int o = q / (kCi * kTaps), r = q - o * (kCi * kTaps), i = r / kTaps, k = r - i * kTaps;
            ws[q] = i < nci ? ld_w(w + ((size_t)o * cin + c0 + i) * kTaps + k) : 0.f;
        }
        for (int q = threadIdx.x; q < kCi * (kTile + 2 * kPad); q += blockDim.x) {
            const int i = q / (kTile + 2 * kPad), ll = q - i * (kTile + 2 * kPad), l = l0 - kPad + ll;
            xs[i * kXPitch + ll] = (i < nci && l >= 0 && l < L) ? inb[(size_t)(c0 + i) * L + l] : 0.f;
        }
        __syncthreads();
#pragma unroll 2
        for (int i = 0; i < kCi; ++i) {
            if (i >= nci) break;   // a pass with fewer channels (the output layer's data gradient has one)
#pragma unroll
            for (int k = 0; k < kTaps; ++k) {
                float xv[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) xv[j] = xs[i * kXPitch + lane + 32 * j + k];
#pragma unroll
                for (int o = 0; o < 8; ++o) {
                    const float wv = ws[((o0 + o) * kCi + i) * kTaps + k];
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[o][j] = fmaf(wv, xv[j], acc[o][j]);
                }
            }
        }
    }
#pragma unroll
    for (int o = 0; o < 8; ++o) {
        const int oc = o0 + o;
        const float bv = bias ? bias[oc] : 0.f;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int l = l0 + lane + 32 * j;
            if (l >= L) continue;
            const size_t idx = ((size_t)e * kHid + oc) * L + l;
            float v = acc[o][j] + bv;
            if (relu) v = fmaxf(v, 0.f);
            if (mask && !(mask[idx] > 0.f)) v = 0.f;
            out[idx] = v;
        }
    }
}

// The output layer: out[e][l] = bias[0] + sum_i sum_k w[i][k] in[e][i][l + k - 3], cin <= 64.
template <typename WT>
__global__ void __launch_bounds__(256) conv1_kernel(const float* __restrict__ in, int cin, int L,
                                                    const WT* __restrict__ w, const float* __restrict__ bias,
                                                    float* __restrict__ out) {
    __shared__ float ws[kHid * kTaps];
    for (int q = threadIdx.x; q < cin * kTaps; q += blockDim.x) ws[q] = ld_w(w + q);
    __syncthreads();
    const int e = blockIdx.y, l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= L) return;
    const float* inb = in + (size_t)e * cin * L;
    float acc = 0.f;
    for (int i = 0; i < cin; ++i)
#pragma unroll
        for (int k = 0; k < kTaps; ++k) {
            const int ll = l + k - kPad;
            if (ll >= 0 && ll < L) acc = fmaf(ws[i * kTaps + k], inb[(size_t)i * L + ll], acc);
        }
    out[(size_t)e * L + l] = acc + bias[0];
}

// Per (example, window): z = the window's largest logit (first maximum); with labels, the
// binary cross-entropy term and, at the maximum's sample, the gradient of the mean loss
// (dlogit zeroed by the caller).
__global__ void window_loss_kernel(const float* __restrict__ logit, int E, int L, int nt, int nwin,
                                   const uint8_t* __restrict__ labels, float inv_n, float* __restrict__ z_out,
                                   float* __restrict__ term, float* __restrict__ dlogit) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= E * nwin) return;
    const int e = idx / nwin, w = idx - e * nwin;
    const int lo = nt + kWin * w, hi = min(lo + kWin, L - nt);
    const float* lr = logit + (size_t)e * L;
    float z = lr[lo];
    int arg = lo;
    for (int l = lo + 1; l < hi; ++l) {
        const float v = lr[l];
        if (v > z) z = v, arg = l;
    }
    if (z_out) z_out[idx] = z;
    if (labels) {
        const float y = labels[idx] ? 1.f : 0.f;
        const float ez = expf(-fabsf(z));
        term[idx] = fmaxf(z, 0.f) + log1pf(ez) - y * z;
        const float sig = z >= 0.f ? 1.f / (1.f + ez) : ez / (1.f + ez);
        dlogit[(size_t)e * L + arg] = (sig - y) * inv_n;
    }
}

// out[0] = scale * (sum of v[0..n) in a fixed order) (one block).
__global__ void __launch_bounds__(256) sum_kernel(const float* __restrict__ v, int n, float scale,
                                                  float* __restrict__ out) {
    __shared__ float red[256];
    float s = 0.f;
    for (int i = threadIdx.x; i < n; i += 256) s += v[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = red[0] * scale;
}

// wt[i][o][k] = w[o][i][6 - k]: the data gradient of a layer as a forward convolution,
//   d in[i][l] = sum_o sum_k w[o][i][k] g[o][l - k + 3] = sum_o sum_k' wt[i][o][k'] g[o][l + k' - 3].
__global__ void flip_kernel(const float* __restrict__ w, int O, int I, float* __restrict__ wt) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= O * I * kTaps) return;
    const int o = q / (I * kTaps), r = q - o * I * kTaps, i = r / kTaps, k = r - i * kTaps;
    wt[((size_t)i * O + o) * kTaps + (kTaps - 1 - k)] = w[q];
}

// Partial gradients of one slice of one example's samples for 8 output channels (slice z of
// gridDim.z, samples [z * Ls, (z + 1) * Ls), written as partial p = e * gridDim.z + z):
//   pw[p][o][i][k] = sum_l g[e][o][l] a[e][i][l + k - 3],   pb[p][o] = sum_l g[e][o][l].
// Thread p owns the (o, i) pairs p, p + 256, ...; a register window slides along the samples.
template <int CIN>
__global__ void __launch_bounds__(256) wgrad_kernel(const float* __restrict__ g, int cout, const float* __restrict__ a,
                                                    int L, int Ls, float* __restrict__ pw, float* __restrict__ pb) {
    constexpr int kPairs = 8 * CIN, R = (kPairs + 255) / 256;
    __shared__ float gs[8][kTile];
    __shared__ float as[CIN * kXPitch];
    const int e = blockIdx.y, og = blockIdx.x * 8, tid = threadIdx.x;
    const int part = e * gridDim.z + blockIdx.z;
    const int lbeg = blockIdx.z * Ls, lend = min(L, lbeg + Ls);
    float acc[R][kTaps];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int k = 0; k < kTaps; ++k) acc[r][k] = 0.f;
    float bacc = 0.f;
    const float* gb = g + (size_t)e * cout * L;
    const float* ab = a + (size_t)e * CIN * L;
    for (int l0 = lbeg; l0 < lend; l0 += kTile) {
        __syncthreads();
        for (int q = tid; q < 8 * kTile; q += 256) {
            const int o = q / kTile, ll = q - o * kTile, l = l0 + ll;
            gs[o][ll] = (og + o < cout && l < lend) ? gb[(size_t)(og + o) * L + l] : 0.f;
        }
        for (int q = tid; q < CIN * (kTile + 2 * kPad); q += 256) {
            const int i = q / (kTile + 2 * kPad), ll = q - i * (kTile + 2 * kPad), l = l0 - kPad + ll;
            as[i * kXPitch + ll] = (l >= 0 && l < L) ? ab[(size_t)i * L + l] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int p = tid + 256 * r;
            if (p < kPairs) {
                const int o = p / CIN, i = p - o * CIN;
                const float* ar = as + i * kXPitch;
                const float* gr = gs[o];
                float x0 = ar[0], x1 = ar[1], x2 = ar[2], x3 = ar[3], x4 = ar[4], x5 = ar[5];
                for (int ll = 0; ll < kTile; ++ll) {
                    const float x6 = ar[ll + 6], gv = gr[ll];
                    acc[r][0] = fmaf(gv, x0, acc[r][0]);
                    acc[r][1] = fmaf(gv, x1, acc[r][1]);
                    acc[r][2] = fmaf(gv, x2, acc[r][2]);
                    acc[r][3] = fmaf(gv, x3, acc[r][3]);
                    acc[r][4] = fmaf(gv, x4, acc[r][4]);
                    acc[r][5] = fmaf(gv, x5, acc[r][5]);
                    acc[r][6] = fmaf(gv, x6, acc[r][6]);
                    x0 = x1, x1 = x2, x2 = x3, x3 = x4, x4 = x5, x5 = x6;
                }
            }
        }
        if (tid < 8)
            for (int ll = 0; ll < kTile; ++ll) bacc += gs[tid][ll];
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int p = tid + 256 * r;
        if (p < kPairs) {
            const int o = p / CIN, i = p - o * CIN;
            if (og + o < cout)
#pragma unroll
                for (int k = 0; k < kTaps; ++k) pw[(((size_t)part * cout + og + o) * CIN + i) * kTaps + k] = acc[r][k];
        }
    }
    if (tid < 8 && og + tid < cout) pb[(size_t)part * cout + og + tid] = bacc;
}

// out[j] = sum_e part[e][j], examples in order.
__global__ void sum_examples_kernel(const float* __restrict__ part, int E, int n, float* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    float s = 0.f;
    for (int e = 0; e < E; ++e) s += part[(size_t)e * n + j];
    out[j] = s;
}

__global__ void adam_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, int n, float lr, float b1, float omb1, float b2, float omb2,
                            float eps, float c1, float c2) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const float gj = g[j];
    const float mj = b1 * m[j] + omb1 * gj;
    const float vj = b2 * v[j] + omb2 * (gj * gj);
    m[j] = mj;
    v[j] = vj;
    p[j] = p[j] - lr * (mj * c1) / (sqrtf(vj * c2) + eps);
}

// open[e][w] = 1 when the window's largest logit exceeds thr.
__global__ void window_open_kernel(const float* __restrict__ logit, int E, int L, int nt, int nwin, float thr,
                                   uint8_t* __restrict__ open) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= E * nwin) return;
    const int e = idx / nwin, w = idx - e * nwin;
    const int lo = nt + kWin * w, hi = min(lo + kWin, L - nt);
    const float* lr = logit + (size_t)e * L;
    float z = lr[lo];
    for (int l = lo + 1; l < hi; ++l) z = fmaxf(z, lr[l]);
    open[idx] = z > thr ? 1 : 0;
}

// dil[e][w] = OR of open[e][w - d .. w + d]; the number of open cells is added to *n_open.
__global__ void __launch_bounds__(256) dilate_kernel(const uint8_t* __restrict__ open, int rows, int nwin, int d,
                                                     uint8_t* __restrict__ dil, unsigned long long* __restrict__ n_open) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = idx < rows * nwin;
    bool v = false;
    if (in) {
        const int e = idx / nwin, w = idx - e * nwin;
        for (int ww = max(0, w - d); ww <= min(nwin - 1, w + d); ++ww) v = v || open[(size_t)e * nwin + ww];
        dil[idx] = v ? 1 : 0;
    }
    const unsigned b = __ballot_sync(0xffffffffu, in && v);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(n_open, (unsigned long long)__popc(b));
}

// Bt[b][s][t] = -1e30 at interior samples s whose cell (owner[t], (s - nt) / 32) is closed.
__global__ void __launch_bounds__(256) gate_scores_kernel(float* __restrict__ Bt, int W, int T, int nt,
                                                          const uint8_t* __restrict__ dil, int NB, int nwin,
                                                          const int* __restrict__ owner) {
    const int b = blockIdx.y;
    const size_t n = (size_t)(W - 2 * nt) * T;
    const uint8_t* db = dil + (size_t)b * NB * nwin;
    float* Bb = Bt + ((size_t)b * W + nt) * T;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(q / T), t = (int)(q - (size_t)r * T);
        if (!db[(size_t)owner[t] * nwin + r / kWin]) Bb[q] = -1e30f;
    }
}

inline int cdiv(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

template <typename WT>
void launch_forward(const float* x, const WT* w, const float* bias, float* a, float* b, float* logit, int E, int L,
                    cudaStream_t st) {
    const dim3 g64(cdiv(L, kTile), E), g1(cdiv(L, 256), E);
    conv64_kernel<WT><<<g64, 256, 0, st>>>(x, kNbc, L, w + kLayers[0].w, bias + kLayers[0].b, nullptr, 1, a);
    conv64_kernel<WT><<<g64, 256, 0, st>>>(a, kHid, L, w + kLayers[1].w, bias + kLayers[1].b, nullptr, 1, b);
    conv64_kernel<WT><<<g64, 256, 0, st>>>(b, kHid, L, w + kLayers[2].w, bias + kLayers[2].b, nullptr, 1, a);
    conv1_kernel<WT><<<g1, 256, 0, st>>>(a, kHid, L, w + kLayers[3].w, bias + kLayers[3].b, logit);
}

}  // namespace

void neighbourhood_starts(int C, std::vector<int32_t>& s) {
    s.clear();
    if (C <= kNbc) {
        s.push_back(0);
        return;
    }
    for (int c = 0; c + kNbc <= C; c += kNbc / 2) s.push_back(c);
    if (s.back() != C - kNbc) s.push_back(C - kNbc);
}

void template_owner(const float* wall3, int T, int K, int C, int32_t* owner) {
    std::vector<int32_t> st;
    neighbourhood_starts(C, st);
    std::vector<int32_t> chan_owner(C);
    for (int c = 0; c < C; ++c) {
        int best = 0;
        double bd = 1e300;
        for (size_t n = 0; n < st.size(); ++n) {
            const double d = std::fabs(c - (st[n] + (kNbc - 1) / 2.0));
            if (d < bd) bd = d, best = (int)n;
        }
        chan_owner[c] = best;
    }
    std::vector<double> en(C);
    for (int t = 0; t < T; ++t) {
        std::fill(en.begin(), en.end(), 0.0);
        for (int k = 0; k < K; ++k)
            for (int c = 0; c < C; ++c) {
                const double v = wall3[((size_t)t * K + k) * C + c];
                en[c] += v * v;
            }
        owner[t] = chan_owner[std::max_element(en.begin(), en.end()) - en.begin()];
    }
}

// ------------------------------------------------------------------------------- sorter gate

struct PropGate {
    int dev = 0, C = 0, T = 0, NB = 0, dil = 0;
    float thr = 0.f;
    std::vector<int32_t> starts;
    __nv_bfloat16* w = nullptr;   // BF16 copy of the parameters (the weights are read from it)
    float* pf = nullptr;          // FP32 copy (the biases are read from it)
    int* owner = nullptr;         // [T]
    int2* pairs = nullptr;        // [chunk * NB] (window within the chunk, neighbourhood start)
    float *x = nullptr, *a = nullptr, *b = nullptr, *logit = nullptr;
    uint8_t *open = nullptr, *dilm = nullptr;
    unsigned long long* n_open = nullptr;
    int chunk = 0, Wcap = 0, nbcap = 0;
    int64_t cells = 0;

    void free_work() {
        for (void* p : {(void*)pairs, (void*)x, (void*)a, (void*)b, (void*)logit, (void*)open, (void*)dilm})
            if (p) cudaFree(p);
        pairs = nullptr, x = a = b = logit = nullptr, open = dilm = nullptr;
        Wcap = nbcap = chunk = 0;
    }
    ~PropGate() {
        free_work();
        for (void* p : {(void*)w, (void*)pf, (void*)owner, (void*)n_open})
            if (p) cudaFree(p);
    }
    template <typename T_>
    T_* alloc(size_t n) {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T_)) != cudaSuccess)
            throw LoadError{LSS_ERR_NOMEM, "proposal gate: device allocation failed"};
        return static_cast<T_*>(p);
    }
    void ensure(int W, int nb, cudaStream_t st) {
        if (W <= Wcap && nb <= nbcap) return;
        PROP_CUDA(cudaStreamSynchronize(st));   // earlier groups may still read the old buffers
        free_work();
        const size_t per_window = (size_t)NB * kHid * W * sizeof(float);
        chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)nb, kGateBytes / per_window));
        chunk = std::min(chunk, std::max(1, 65535 / NB));
        const size_t E = (size_t)chunk * NB;
        pairs = alloc<int2>(E);
        x = alloc<float>(E * kNbc * W);
        a = alloc<float>(E * kHid * W);
        b = alloc<float>(E * kHid * W);
        logit = alloc<float>(E * W);
        const size_t cells_cap = (size_t)nb * NB * cdiv(W, kWin);
        open = alloc<uint8_t>(cells_cap);
        dilm = alloc<uint8_t>(cells_cap);
        std::vector<int2> hp(E);
        for (size_t e = 0; e < E; ++e) hp[e] = make_int2((int)(e / NB), starts[e % NB]);
        PROP_CUDA(cudaMemcpy(pairs, hp.data(), E * sizeof(int2), cudaMemcpyHostToDevice));
        Wcap = W, nbcap = nb;
    }
};

PropGate* prop_gate_create(int device, const float* params, float logit_threshold, int dilate, const float* wall3,
                           int T, int K, int C) {
    if (dilate < 0) throw LoadError{LSS_ERR_ARG, "proposal gate: dilate must be >= 0"};
    for (int j = 0; j < LSS_PROP_N_PARAMS; ++j)
        if (!std::isfinite(params[j])) throw LoadError{LSS_ERR_ARG, "proposal gate: parameters must be finite"};
    PropGate* g = new PropGate;
    try {
        g->dev = device, g->C = C, g->T = T, g->thr = logit_threshold, g->dil = dilate;
        neighbourhood_starts(C, g->starts);
        g->NB = (int)g->starts.size();
        std::vector<int32_t> own(T);
        template_owner(wall3, T, K, C, own.data());
        std::vector<__nv_bfloat16> wb(LSS_PROP_N_PARAMS);
        for (int j = 0; j < LSS_PROP_N_PARAMS; ++j) wb[j] = __float2bfloat16_rn(params[j]);
        g->w = g->alloc<__nv_bfloat16>(LSS_PROP_N_PARAMS);
        g->pf = g->alloc<float>(LSS_PROP_N_PARAMS);
        g->owner = g->alloc<int>(T);
        g->n_open = g->alloc<unsigned long long>(1);
        PROP_CUDA(cudaMemcpy(g->w, wb.data(), wb.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice));
        PROP_CUDA(cudaMemcpy(g->pf, params, LSS_PROP_N_PARAMS * sizeof(float), cudaMemcpyHostToDevice));
        PROP_CUDA(cudaMemcpy(g->owner, own.data(), T * sizeof(int), cudaMemcpyHostToDevice));
        PROP_CUDA(cudaMemset(g->n_open, 0, sizeof(unsigned long long)));
    } catch (const CudaFail& e) {
        delete g;
        throw LoadError{LSS_ERR_CUDA, e.msg};
    } catch (...) {
        delete g;
        throw;
    }
    return g;
}

void prop_gate_destroy(PropGate* g) { delete g; }

int prop_gate_run(PropGate* g, const float* Z, float* Bt, int nb, int W, int nt, cudaStream_t st) {
    try {
        g->ensure(W, nb, st);
    } catch (const CudaFail& e) {
        throw LoadError{LSS_ERR_CUDA, e.msg};
    }
    const int nwin = cdiv(W - 2 * nt, kWin);
    int launches = 0;
    for (int b0 = 0; b0 < nb; b0 += g->chunk) {
        const int nbc = std::min(g->chunk, nb - b0), E = nbc * g->NB;
        gather_kernel<<<dim3(cdiv(W, 64), E), 256, 0, st>>>(Z + (size_t)b0 * W * g->C, W, g->C, g->pairs, g->x);
        launch_forward(g->x, g->w, g->pf, g->a, g->b, g->logit, E, W, st);
        window_open_kernel<<<cdiv((int64_t)E * nwin, 256), 256, 0, st>>>(g->logit, E, W, nt, nwin, g->thr,
                                                                          g->open + (size_t)b0 * g->NB * nwin);
        launches += 6;
    }
    const int rows = nb * g->NB;
    dilate_kernel<<<cdiv((int64_t)rows * nwin, 256), 256, 0, st>>>(g->open, rows, nwin, g->dil, g->dilm, g->n_open);
    const int gx = std::min(1024, cdiv((int64_t)(W - 2 * nt) * g->T, 256));
    gate_scores_kernel<<<dim3(gx, nb), 256, 0, st>>>(Bt, W, g->T, nt, g->dilm, g->NB, nwin, g->owner);
    g->cells += (int64_t)rows * nwin;
    return launches + 2;
}

void prop_gate_stats(PropGate* g, cudaStream_t st, int64_t* cells, int64_t* open) {
    unsigned long long n = 0;
    if (cudaStreamSynchronize(st) != cudaSuccess ||
        cudaMemcpy(&n, g->n_open, sizeof(n), cudaMemcpyDeviceToHost) != cudaSuccess)
        throw LoadError{LSS_ERR_CUDA, "proposal gate: reading its counters failed"};
    *cells = g->cells;
    *open = (int64_t)n;
}

}  // namespace lss

// ------------------------------------------------------------------------------- trainer

struct lss_prop_trainer {
    int dev = 0;
    cudaStream_t st = nullptr;
    int maxE = 0, W = 0, nt = 0, nwin = 0;
    float lr = 1e-3f, b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    int64_t step = 0;
    float *p = nullptr, *m = nullptr, *v = nullptr, *g = nullptr, *wt = nullptr;
    float *x = nullptr, *a1 = nullptr, *a2 = nullptr, *a3 = nullptr, *logit = nullptr, *dlogit = nullptr;
    float *ga = nullptr, *gb = nullptr, *pw = nullptr, *pb = nullptr, *z = nullptr, *term = nullptr, *loss = nullptr;
    int2* pairs = nullptr;
    uint8_t* labels = nullptr;
    std::string err;

    ~lss_prop_trainer() {
        if (st) cudaStreamSynchronize(st);
        for (void* q : {(void*)p, (void*)m, (void*)v, (void*)g, (void*)wt, (void*)x, (void*)a1, (void*)a2, (void*)a3,
                        (void*)logit, (void*)dlogit, (void*)ga, (void*)gb, (void*)pw, (void*)pb, (void*)z,
                        (void*)term, (void*)loss, (void*)pairs, (void*)labels})
            if (q) cudaFree(q);
        if (st) cudaStreamDestroy(st);
    }
};

namespace {
using lss::CudaFail;
using lss::LoadError;

template <typename T_>
T_* talloc(size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T_)) != cudaSuccess)
        throw LoadError{LSS_ERR_NOMEM, "trainer: device allocation failed"};
    return static_cast<T_*>(q);
}

// Copy the examples' (window, start) pairs and labels to the device and build x.
void stage_examples(lss_prop_trainer* tr, const float* z_dev, int32_t n_windows, int32_t C, const int32_t* pairs,
                    const uint8_t* labels, int32_t E) {
    if (!z_dev || !pairs || n_windows <= 0 || C <= 0 || E <= 0 || E > tr->maxE)
        throw LoadError{LSS_ERR_ARG, "trainer: bad examples (E must be in [1, max_examples])"};
    std::vector<int2> hp(E);
    for (int e = 0; e < E; ++e) {
        const int j = pairs[2 * e], c0 = pairs[2 * e + 1];
        const bool ok_c = C <= lss::kNbc ? c0 == 0 : (c0 >= 0 && c0 + lss::kNbc <= C);
        if (j < 0 || j >= n_windows || !ok_c) throw LoadError{LSS_ERR_ARG, "trainer: example pair out of range"};
        hp[e] = make_int2(j, c0);
    }
    PROP_CUDA(cudaMemcpyAsync(tr->pairs, hp.data(), E * sizeof(int2), cudaMemcpyHostToDevice, tr->st));
    if (labels)
        PROP_CUDA(cudaMemcpyAsync(tr->labels, labels, (size_t)E * tr->nwin, cudaMemcpyHostToDevice, tr->st));
    lss::gather_kernel<<<dim3(lss::cdiv(tr->W, 64), E), 256, 0, tr->st>>>(z_dev, tr->W, C, tr->pairs, tr->x);
    // the host vectors must outlive the copies
    PROP_CUDA(cudaStreamSynchronize(tr->st));
}

void forward(lss_prop_trainer* tr, int E) {
    lss::launch_forward<float>(tr->x, tr->p, tr->p, tr->a1, tr->a2, tr->logit, E, tr->W, tr->st);
}

// The forward pass keeps a1, a2, a3 for the backward pass (launch_forward ping-pongs two buffers).
void forward_keep(lss_prop_trainer* tr, int E) {
    using namespace lss;
    const int L = tr->W;
    const dim3 g64(cdiv(L, kTile), E), g1(cdiv(L, 256), E);
    conv64_kernel<float><<<g64, 256, 0, tr->st>>>(tr->x, kNbc, L, tr->p + kLayers[0].w, tr->p + kLayers[0].b, nullptr,
                                                  1, tr->a1);
    conv64_kernel<float><<<g64, 256, 0, tr->st>>>(tr->a1, kHid, L, tr->p + kLayers[1].w, tr->p + kLayers[1].b,
                                                  nullptr, 1, tr->a2);
    conv64_kernel<float><<<g64, 256, 0, tr->st>>>(tr->a2, kHid, L, tr->p + kLayers[2].w, tr->p + kLayers[2].b,
                                                  nullptr, 1, tr->a3);
    conv1_kernel<float><<<g1, 256, 0, tr->st>>>(tr->a3, kHid, L, tr->p + kLayers[3].w, tr->p + kLayers[3].b,
                                                tr->logit);
}

void loss_and_backward(lss_prop_trainer* tr, int E) {
    using namespace lss;
    const int L = tr->W, n = E * tr->nwin;
    cudaStream_t st = tr->st;
    PROP_CUDA(cudaMemsetAsync(tr->dlogit, 0, (size_t)E * L * sizeof(float), st));
    window_loss_kernel<<<cdiv(n, 256), 256, 0, st>>>(tr->logit, E, L, tr->nt, tr->nwin, tr->labels, 1.f / n, tr->z,
                                                     tr->term, tr->dlogit);
    sum_kernel<<<1, 256, 0, st>>>(tr->term, n, 1.f / n, tr->loss);   // the mean
    // flipped weights of layers 2..4 at wt + {0, 28672, 57344}
    float* wt2 = tr->wt;
    float* wt3 = tr->wt + kHid * kHid * kTaps;
    float* wt4 = tr->wt + 2 * kHid * kHid * kTaps;
    flip_kernel<<<cdiv(kHid * kHid * kTaps, 256), 256, 0, st>>>(tr->p + kLayers[1].w, kHid, kHid, wt2);
    flip_kernel<<<cdiv(kHid * kHid * kTaps, 256), 256, 0, st>>>(tr->p + kLayers[2].w, kHid, kHid, wt3);
    flip_kernel<<<cdiv(kHid * kTaps, 256), 256, 0, st>>>(tr->p + kLayers[3].w, 1, kHid, wt4);
    const dim3 g64(cdiv(L, kTile), E);
    auto reduce = [&](int li, int cout, int cin, int parts) {
        const int nw = cout * cin * kTaps;
        sum_examples_kernel<<<cdiv(nw, 256), 256, 0, st>>>(tr->pw, parts, nw, tr->g + kLayers[li].w);
        sum_examples_kernel<<<cdiv(cout, 256), 256, 0, st>>>(tr->pb, parts, cout, tr->g + kLayers[li].b);
    };
    // layer 4 (64 -> 1): one output channel, so the samples are split into slices of 256 (at most
    // 64 per example, within the partial buffers' E * 64 rows) to fill the GPU
    const int zs = std::min(64, cdiv(L, 2 * kTile));
    const int ls = cdiv(cdiv(L, zs), kTile) * kTile;
    wgrad_kernel<kHid><<<dim3(1, E, zs), 256, 0, st>>>(tr->dlogit, 1, tr->a3, L, ls, tr->pw, tr->pb);
    reduce(3, 1, kHid, E * zs);
    conv64_kernel<float><<<g64, 256, 0, st>>>(tr->dlogit, 1, L, wt4, nullptr, tr->a3, 0, tr->ga);
    // layer 3
    wgrad_kernel<kHid><<<dim3(kHid / 8, E, 1), 256, 0, st>>>(tr->ga, kHid, tr->a2, L, L, tr->pw, tr->pb);
    reduce(2, kHid, kHid, E);
    conv64_kernel<float><<<g64, 256, 0, st>>>(tr->ga, kHid, L, wt3, nullptr, tr->a2, 0, tr->gb);
    // layer 2
    wgrad_kernel<kHid><<<dim3(kHid / 8, E, 1), 256, 0, st>>>(tr->gb, kHid, tr->a1, L, L, tr->pw, tr->pb);
    reduce(1, kHid, kHid, E);
    conv64_kernel<float><<<g64, 256, 0, st>>>(tr->gb, kHid, L, wt2, nullptr, tr->a1, 0, tr->ga);
    // layer 1 (16 -> 64)
    wgrad_kernel<kNbc><<<dim3(kHid / 8, E, 1), 256, 0, st>>>(tr->ga, kHid, tr->x, L, L, tr->pw, tr->pb);
    reduce(0, kHid, kNbc, E);
    PROP_CUDA(cudaGetLastError());
}

}  // namespace

#define PROP_TRY(tr, ...)                                                                          \
    try {                                                                                          \
        PROP_CUDA(cudaSetDevice((tr)->dev));                                                       \
        __VA_ARGS__;                                                                               \
        return LSS_OK;                                                                             \
    } catch (const lss::LoadError& e) {                                                            \
        (tr)->err = e.msg;                                                                         \
        return e.status;                                                                           \
    } catch (const lss::CudaFail& e) {                                                             \
        (tr)->err = e.msg;                                                                         \
        return LSS_ERR_CUDA;                                                                       \
    } catch (const std::exception& e) {                                                            \
        (tr)->err = e.what();                                                                      \
        return LSS_ERR_INTERNAL;                                                                   \
    }

extern "C" {

int lss_prop_neighbourhoods(int32_t n_chan, int32_t* n_nbhd, int32_t* starts, int32_t cap) {
    if (n_chan <= 0 || !n_nbhd || cap < 0 || (cap > 0 && !starts)) return LSS_ERR_ARG;
    std::vector<int32_t> s;
    lss::neighbourhood_starts(n_chan, s);
    *n_nbhd = (int32_t)s.size();
    for (int i = 0; i < std::min<int>(cap, (int)s.size()); ++i) starts[i] = s[i];
    return LSS_OK;
}

int lss_prop_template_owner(const float* wall3, int32_t T, int32_t K, int32_t C, int32_t* owner) {
    if (!wall3 || !owner || T <= 0 || K <= 0 || C <= 0) return LSS_ERR_ARG;
    lss::template_owner(wall3, T, K, C, owner);
    return LSS_OK;
}

int lss_prop_trainer_open(const lss_prop_train_params* p, const float* init_params, lss_prop_trainer** out) {
    if (!p || !init_params || !out) return LSS_ERR_ARG;
    *out = nullptr;
    if (p->max_examples <= 0 || p->max_examples > 65535 || p->nt < 0 || p->W <= 2 * p->nt + 1) return LSS_ERR_ARG;
    lss_prop_trainer* tr = new (std::nothrow) lss_prop_trainer;
    if (!tr) return LSS_ERR_NOMEM;
    tr->dev = p->device;
    tr->maxE = p->max_examples, tr->W = p->W, tr->nt = p->nt;
    tr->nwin = lss::cdiv(p->W - 2 * p->nt, lss::kWin);
    if (p->lr > 0) tr->lr = p->lr;
    if (p->beta1 > 0) tr->b1 = p->beta1;
    if (p->beta2 > 0) tr->b2 = p->beta2;
    if (p->eps > 0) tr->eps = p->eps;
    auto body = [&]() {
        PROP_CUDA(cudaStreamCreateWithFlags(&tr->st, cudaStreamNonBlocking));
        const size_t E = tr->maxE, L = tr->W, N = LSS_PROP_N_PARAMS;
        tr->p = talloc<float>(N), tr->m = talloc<float>(N), tr->v = talloc<float>(N), tr->g = talloc<float>(N);
        tr->wt = talloc<float>(2 * lss::kHid * lss::kHid * lss::kTaps + lss::kHid * lss::kTaps);
        tr->x = talloc<float>(E * lss::kNbc * L);
        tr->a1 = talloc<float>(E * lss::kHid * L), tr->a2 = talloc<float>(E * lss::kHid * L);
        tr->a3 = talloc<float>(E * lss::kHid * L);
        tr->ga = talloc<float>(E * lss::kHid * L), tr->gb = talloc<float>(E * lss::kHid * L);
        tr->logit = talloc<float>(E * L), tr->dlogit = talloc<float>(E * L);
        tr->pw = talloc<float>(E * lss::kHid * lss::kHid * lss::kTaps), tr->pb = talloc<float>(E * lss::kHid);
        tr->z = talloc<float>(E * tr->nwin), tr->term = talloc<float>(E * tr->nwin), tr->loss = talloc<float>(1);
        tr->pairs = talloc<int2>(E), tr->labels = talloc<uint8_t>(E * tr->nwin);
        PROP_CUDA(cudaMemcpy(tr->p, init_params, N * sizeof(float), cudaMemcpyHostToDevice));
        PROP_CUDA(cudaMemset(tr->m, 0, N * sizeof(float)));
        PROP_CUDA(cudaMemset(tr->v, 0, N * sizeof(float)));
    };
    int st = LSS_OK;
    try {
        PROP_CUDA(cudaSetDevice(tr->dev));
        body();
    } catch (const lss::LoadError& e) {
        lss::g_handleless_error = e.msg;
        st = e.status;
    } catch (const lss::CudaFail& e) {
        lss::g_handleless_error = e.msg;
        st = LSS_ERR_CUDA;
    }
    if (st != LSS_OK) {
        delete tr;
        return st;
    }
    *out = tr;
    return LSS_OK;
}

int lss_prop_trainer_close(lss_prop_trainer* tr) {
    if (!tr) return LSS_ERR_ARG;
    cudaSetDevice(tr->dev);
    delete tr;
    return LSS_OK;
}

const char* lss_prop_trainer_last_error(const lss_prop_trainer* tr) {
    return tr ? tr->err.c_str() : lss::g_handleless_error.c_str();
}

int lss_prop_train_step(lss_prop_trainer* tr, const float* z_dev, int32_t n_windows, int32_t C, const int32_t* pairs,
                        const uint8_t* labels, int32_t E, float* loss) {
    if (!tr) return LSS_ERR_ARG;
    PROP_TRY(tr, {
        if (!labels) throw LoadError{LSS_ERR_ARG, "trainer: labels required"};
        stage_examples(tr, z_dev, n_windows, C, pairs, labels, E);
        forward_keep(tr, E);
        loss_and_backward(tr, E);
        ++tr->step;
        const double c1 = 1.0 / (1.0 - std::pow((double)tr->b1, (double)tr->step));
        const double c2 = 1.0 / (1.0 - std::pow((double)tr->b2, (double)tr->step));
        lss::adam_kernel<<<lss::cdiv(LSS_PROP_N_PARAMS, 256), 256, 0, tr->st>>>(
            tr->p, tr->m, tr->v, tr->g, LSS_PROP_N_PARAMS, tr->lr, tr->b1, (float)(1.0 - (double)tr->b1), tr->b2,
            (float)(1.0 - (double)tr->b2), tr->eps, (float)c1, (float)c2);
        PROP_CUDA(cudaGetLastError());
        float l = 0.f;
        PROP_CUDA(cudaMemcpyAsync(&l, tr->loss, sizeof(float), cudaMemcpyDeviceToHost, tr->st));
        PROP_CUDA(cudaStreamSynchronize(tr->st));
        if (loss) *loss = l;
    })
}

int lss_prop_loss_grad(lss_prop_trainer* tr, const float* z_dev, int32_t n_windows, int32_t C, const int32_t* pairs,
                       const uint8_t* labels, int32_t E, float* loss, float* grad) {
    if (!tr) return LSS_ERR_ARG;
    PROP_TRY(tr, {
        if (!labels) throw LoadError{LSS_ERR_ARG, "trainer: labels required"};
        stage_examples(tr, z_dev, n_windows, C, pairs, labels, E);
        forward_keep(tr, E);
        loss_and_backward(tr, E);
        float l = 0.f;
        PROP_CUDA(cudaMemcpyAsync(&l, tr->loss, sizeof(float), cudaMemcpyDeviceToHost, tr->st));
        if (grad)
            PROP_CUDA(cudaMemcpyAsync(grad, tr->g, LSS_PROP_N_PARAMS * sizeof(float), cudaMemcpyDeviceToHost, tr->st));
        PROP_CUDA(cudaStreamSynchronize(tr->st));
        if (loss) *loss = l;
    })
}

int lss_prop_forward(lss_prop_trainer* tr, const float* z_dev, int32_t n_windows, int32_t C, const int32_t* pairs,
                     int32_t E, float* logits, float* window_logits) {
    if (!tr) return LSS_ERR_ARG;
    PROP_TRY(tr, {
        stage_examples(tr, z_dev, n_windows, C, pairs, nullptr, E);
        forward(tr, E);
        const int n = E * tr->nwin;
        lss::window_loss_kernel<<<lss::cdiv(n, 256), 256, 0, tr->st>>>(tr->logit, E, tr->W, tr->nt, tr->nwin, nullptr,
                                                                        0.f, tr->z, nullptr, nullptr);
        PROP_CUDA(cudaGetLastError());
        if (logits)
            PROP_CUDA(cudaMemcpyAsync(logits, tr->logit, (size_t)E * tr->W * sizeof(float), cudaMemcpyDeviceToHost,
                                      tr->st));
        if (window_logits)
            PROP_CUDA(cudaMemcpyAsync(window_logits, tr->z, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, tr->st));
        PROP_CUDA(cudaStreamSynchronize(tr->st));
    })
}

int lss_prop_get_params(lss_prop_trainer* tr, float* params) {
    if (!tr || !params) return LSS_ERR_ARG;
    PROP_TRY(tr, {
        PROP_CUDA(cudaMemcpyAsync(params, tr->p, LSS_PROP_N_PARAMS * sizeof(float), cudaMemcpyDeviceToHost, tr->st));
        PROP_CUDA(cudaStreamSynchronize(tr->st));
    })
}

int lss_prop_set_params(lss_prop_trainer* tr, const float* params) {
    if (!tr || !params) return LSS_ERR_ARG;
    PROP_TRY(tr, {
        PROP_CUDA(cudaMemcpyAsync(tr->p, params, LSS_PROP_N_PARAMS * sizeof(float), cudaMemcpyHostToDevice, tr->st));
        PROP_CUDA(cudaMemsetAsync(tr->m, 0, LSS_PROP_N_PARAMS * sizeof(float), tr->st));
        PROP_CUDA(cudaMemsetAsync(tr->v, 0, LSS_PROP_N_PARAMS * sizeof(float), tr->st));
        PROP_CUDA(cudaStreamSynchronize(tr->st));
        tr->step = 0;
    })
}

}  // extern "C"
