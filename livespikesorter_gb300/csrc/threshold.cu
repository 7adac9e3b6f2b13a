// threshold.cu -- the threshold-crossing detector (the reference's ThresholdCrossing sorter,
// src/SpikeSorter/ThresholdCrossing.cpp:112-252) on the GPU, behind include/lss_threshold.h.
//
// The reference tests, for each channel c and row j of a fetched block,
//     (double)((float)x - means[c]) <= -1.0 * (double)threshold_std * (double)medians[c]
// (ThresholdCrossing.cpp:209-226).  (float)x - m is monotone in x, so the test equals x <= X[c]
// for one integer X[c] per channel, found on the host by bisection over the int16 range with the
// same float arithmetic.  The device work is then a pure int16 stream compare, HBM-bound:
//
//   count   one pass over the rows.  A thread owns one unit = V adjacent channels (V = 8: one
//           16-byte load per row) x S consecutive rows; it counts its crossings per channel and
//           keeps the first kKeep of them as packed (row, channel, sample) words.  A CTA holds
//           R units of consecutive slabs over all channel groups and writes its per-channel totals.
//   offsets per channel, the exclusive prefix of the CTA totals along the rows and the total.
//   emit    per CTA: the channel prefix of the totals (the reference emits channel by channel),
//           the CTA's per-unit counts (from the kept words; a unit with more than kKeep crossings
//           reads its rows again) scanned along its slabs, then every unit writes its events, rows
//           in order per channel, as 16-byte records into device memory.
//   copy    the events, contiguous, into host-mapped memory (coalesced 16-byte writes over the
//           CPU-GPU link; the scattered writes of the emit pass stay in HBM).
//
// Input traffic is 2 bytes per channel-sample once; the offsets pass moves C ints per CTA; the
// events cost 16 bytes each written and read in HBM and 16 bytes each to the host.
#include "../../include/lss_threshold.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <new>
#include <string>
#include <vector>

namespace lss {
void par_memcpy(void* dst, const void* src, size_t bytes);   // sorter.cu
extern thread_local std::string g_handleless_error;
}

namespace lss {
namespace tc {

constexpr int kKeep = 32;            // crossings a unit keeps from the count pass
constexpr int kUnitsPerCta = 512;    // R x G <= this (threads per CTA)
constexpr int kMinSlab = 16, kMaxSlab = 32;    // <= 256 channel-samples per unit
constexpr int64_t kFillUnits = 152LL * 1024;   // units that fill the GPU (152 SMs x 1024 threads)
constexpr int kSlots = 3;

struct Geometry {
    int V = 1, G = 0, S = kMinSlab, R = 1;
    int64_t nslabs = 0, nctas = 0;
};

// V = channels per thread, G = channel groups, S = rows per unit (power of two, grown while the
// grid still fills the GPU), R = slabs per CTA
static Geometry geometry(int C, int64_t n_rows, int V) {
    Geometry g;
    g.V = V;
    g.G = C / V;
    g.R = std::max(1, kUnitsPerCta / g.G);
    g.S = kMinSlab;
    while (g.S < kMaxSlab && ((n_rows + 2 * g.S - 1) / (2 * g.S)) * g.G >= kFillUnits) g.S *= 2;
    g.nslabs = (n_rows + g.S - 1) / g.S;
    g.nctas = (g.nslabs + g.R - 1) / g.R;
    return g;
}

template <int V>
struct Row;
template <>
struct Row<8> {
    uint4 v;
    __device__ __forceinline__ void load(const int16_t* p) { v = __ldg(reinterpret_cast<const uint4*>(p)); }
    __device__ __forceinline__ int at(int k) const {
        const unsigned w = k < 2 ? v.x : k < 4 ? v.y : k < 6 ? v.z : v.w;
        return (int)(int16_t)(uint16_t)((k & 1) ? (w >> 16) : (w & 0xffffu));
    }
};
template <>
struct Row<1> {
    int16_t v;
    __device__ __forceinline__ void load(const int16_t* p) { v = __ldg(p); }
    __device__ __forceinline__ int at(int) const { return v; }
};

// (row within the unit, channel within the group, sample) in one word
__device__ __forceinline__ uint32_t pack(int r, int k, int x) {
    return ((uint32_t)(r * 8 + k) << 16) | (uint32_t)(uint16_t)(int16_t)x;
}
__device__ __forceinline__ int unpack_r(uint32_t e) { return (int)(e >> 19); }
__device__ __forceinline__ int unpack_k(uint32_t e) { return (int)((e >> 16) & 7u); }
__device__ __forceinline__ int unpack_x(uint32_t e) { return (int)(int16_t)(uint16_t)(e & 0xffffu); }

// bit k set when channel k of the 8 int16 in v is <= its threshold (t: thresholds clamped to
// int16, en: 0xffff where a channel can cross at all, 0 where its threshold is below -32768)
__device__ __forceinline__ unsigned cross_mask8(const uint4& v, const uint4& t, const uint4& en) {
    const unsigned m0 = __vcmples2(v.x, t.x) & en.x, m1 = __vcmples2(v.y, t.y) & en.y;
    const unsigned m2 = __vcmples2(v.z, t.z) & en.z, m3 = __vcmples2(v.w, t.w) & en.w;
    return (m0 & 1u) | ((m0 >> 15) & 2u) | ((m1 & 1u) << 2) | ((m1 >> 13) & 8u) | ((m2 & 1u) << 4) |
           ((m2 >> 11) & 32u) | ((m3 & 1u) << 6) | ((m3 >> 9) & 128u);
}

// count pass, 8 channels per thread: four packed compares per row, the rare crossings recorded on
// a side path; per-channel CTA totals by shared-memory atomics
__global__ void __launch_bounds__(kUnitsPerCta, 2)
tc_count8_kernel(const int16_t* __restrict__ rows, int64_t n_rows, int C, int G, int S, int R, int64_t nslabs,
                 const int16_t* __restrict__ thr16, const uint16_t* __restrict__ en16, uint32_t* __restrict__ ent,
                 int* __restrict__ ucnt, int* __restrict__ ctot) {
    extern __shared__ int s_tot[];   // [C]
    const int tid = threadIdx.x;
    for (int c = tid; c < C; c += blockDim.x) s_tot[c] = 0;
    __syncthreads();
    const int rl = tid / G, g = tid - rl * G;
    const int64_t slab = (int64_t)blockIdx.x * R + rl;
    if (slab < nslabs) {
        const uint4 t = __ldg(reinterpret_cast<const uint4*>(thr16) + g);
        const uint4 en = __ldg(reinterpret_cast<const uint4*>(en16) + g);
        const int64_t r0 = slab * S;
        const int nr = (int)min((int64_t)S, n_rows - r0);
        const uint4* p = reinterpret_cast<const uint4*>(rows + r0 * C) + g;
        const int64_t stride = C / 8;   // uint4 per row
        const int64_t u = slab * G + g;
        uint32_t* e = ent + u * kKeep;
        int kept = 0;
        auto record = [&](const uint4& v, unsigned m, int r) {
            while (m) {
                const int k = __ffs(m) - 1;
                m &= m - 1;
                const unsigned w = k < 2 ? v.x : k < 4 ? v.y : k < 6 ? v.z : v.w;
                const int x = (int)(int16_t)(uint16_t)((k & 1) ? (w >> 16) : (w & 0xffffu));
                atomicAdd(&s_tot[g * 8 + k], 1);
                if (kept < kKeep) e[kept] = pack(r, k, x);
                ++kept;
            }
        };
        int r = 0;
        for (; r + 8 <= nr; r += 8) {
            uint4 v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) v[j] = __ldg(p + (int64_t)(r + j) * stride);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const unsigned m = cross_mask8(v[j], t, en);
                if (m) record(v[j], m, r + j);
            }
        }
        for (; r < nr; ++r) {
            const uint4 v = __ldg(p + (int64_t)r * stride);
            const unsigned m = cross_mask8(v, t, en);
            if (m) record(v, m, r);
        }
        ucnt[u] = kept;
    }
    __syncthreads();
    for (int c = tid; c < C; c += blockDim.x) ctot[(int64_t)blockIdx.x * C + c] = s_tot[c];
}

// count pass, one channel per thread (rows not 16-byte aligned or C not a multiple of 8)
__global__ void __launch_bounds__(kUnitsPerCta, 2)
tc_count1_kernel(const int16_t* __restrict__ rows, int64_t n_rows, int C, int G, int S, int R, int64_t nslabs,
                 const int* __restrict__ thr, uint32_t* __restrict__ ent, int* __restrict__ ucnt,
                 int* __restrict__ ctot) {
    extern __shared__ int s_tot[];   // [C]
    const int tid = threadIdx.x;
    const int rl = tid / G, g = tid - rl * G;
    const int64_t slab = (int64_t)blockIdx.x * R + rl;
    int cnt = 0;
    if (slab < nslabs) {
        const int th = __ldg(thr + g);
        const int64_t r0 = slab * S;
        const int nr = (int)min((int64_t)S, n_rows - r0);
        const int16_t* p = rows + r0 * C + g;
        const int64_t u = slab * G + g;
        uint32_t* e = ent + u * kKeep;
        int r = 0;
        for (; r + 8 <= nr; r += 8) {
            int x[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) x[j] = __ldg(p + (int64_t)(r + j) * C);
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (x[j] <= th) {
                    if (cnt < kKeep) e[cnt] = pack(r + j, 0, x[j]);
                    ++cnt;
                }
        }
        for (; r < nr; ++r) {
            const int x = __ldg(p + (int64_t)r * C);
            if (x <= th) {
                if (cnt < kKeep) e[cnt] = pack(r, 0, x);
                ++cnt;
            }
        }
        ucnt[u] = cnt;
    }
    s_tot[rl * C + g] = cnt;   // [R][C] here: one channel per thread
    __syncthreads();
    for (int c = tid; c < C; c += blockDim.x) {
        int sum = 0;
        for (int i = 0; i < R; ++i) sum += s_tot[i * C + c];
        ctot[(int64_t)blockIdx.x * C + c] = sum;
    }
}

// per channel: ctot[cta][c] <- exclusive prefix along the CTAs, tot[c] <- total
__global__ void __launch_bounds__(1024) tc_offsets_kernel(int* __restrict__ ctot, int64_t nctas, int C,
                                                          int* __restrict__ tot) {
    __shared__ int part[32][33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int c = blockIdx.x * 32 + lane;
    const int64_t per = (nctas + 31) / 32;
    const int64_t a = min(nctas, (int64_t)w * per), b = min(nctas, a + per);
    int s = 0;
    if (c < C)
        for (int64_t i = a; i < b; ++i) s += ctot[i * C + c];
    part[w][lane] = s;
    __syncthreads();
    if (w == 0) {
        int run = 0;
        for (int i = 0; i < 32; ++i) {
            const int t = part[i][lane];
            part[i][lane] = run;
            run += t;
        }
        if (c < C) tot[c] = run;
    }
    __syncthreads();
    if (c < C) {
        int run = part[w][lane];
        for (int64_t i = a; i < b; ++i) {
            const int t = ctot[i * C + c];
            ctot[i * C + c] = run;
            run += t;
        }
    }
}

template <int V>
__global__ void __launch_bounds__(kUnitsPerCta)
tc_emit_kernel(const int16_t* __restrict__ rows, int64_t n_rows, int C, int G, int S, int R, int64_t nslabs,
               const int* __restrict__ thr, const float* __restrict__ means, const uint32_t* __restrict__ ent,
               const int* __restrict__ ucnt, const int* __restrict__ ctoff, const int* __restrict__ tot,
               int64_t first_row, int4* __restrict__ out, int64_t cap, long long* __restrict__ total_out) {
    // out / total_out are device memory; tc_copy_kernel moves the events to the host
    extern __shared__ int smem[];
    int* s_pre = smem;          // [C] events of all channels before c
    int* s_cnt = smem + C;      // [R][C] per-unit counts, then their positions
    const int tid = threadIdx.x, nthr = blockDim.x;
    for (int c = tid; c < C; c += nthr) s_pre[c] = tot[c];
    __syncthreads();
    if (tid < 32) {
        // exclusive scan over the channels: each lane a contiguous chunk, then a warp scan
        const int per = (C + 31) / 32;
        const int a = min(C, tid * per), b = min(C, a + per);
        int s = 0;
        for (int c = a; c < b; ++c) s += s_pre[c];
        int inc = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, inc, o);
            if (tid >= o) inc += v;
        }
        int run = inc - s;
        for (int c = a; c < b; ++c) {
            const int t = s_pre[c];
            s_pre[c] = run;
            run += t;
        }
        if (blockIdx.x == 0 && tid == 31) *total_out = (long long)inc;
    }
    const int rl = tid / G, g = tid - rl * G;
    const int64_t slab = (int64_t)blockIdx.x * R + rl;
    const bool active = slab < nslabs;
    const int64_t u = slab * G + g;
    const int64_t r0 = slab * S;
    const int nr = active ? (int)min((int64_t)S, n_rows - r0) : 0;
    const int16_t* p = rows + r0 * C + g * V;
    int th[V];
#pragma unroll
    for (int k = 0; k < V; ++k) th[k] = active ? __ldg(thr + g * V + k) : 0;
    const int kept = active ? __ldg(ucnt + u) : 0;
    const bool reread = kept > kKeep;
    const uint32_t* e = ent + u * kKeep;
    int cnt[V];
#pragma unroll
    for (int k = 0; k < V; ++k) cnt[k] = 0;
    if (!reread) {
        for (int i = 0; i < kept; ++i) {
            const int kk = unpack_k(__ldg(e + i));
#pragma unroll
            for (int k = 0; k < V; ++k) cnt[k] += (k == kk);
        }
    } else {
        for (int r = 0; r < nr; ++r) {
            Row<V> v;
            v.load(p + (int64_t)r * C);
#pragma unroll
            for (int k = 0; k < V; ++k) cnt[k] += (v.at(k) <= th[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < V; ++k) s_cnt[rl * C + g * V + k] = cnt[k];
    __syncthreads();
    for (int c = tid; c < C; c += nthr) {
        int run = s_pre[c] + ctoff[(int64_t)blockIdx.x * C + c];
        for (int i = 0; i < R; ++i) {
            const int t = s_cnt[i * C + c];
            s_cnt[i * C + c] = run;
            run += t;
        }
    }
    __syncthreads();
    if (!active) return;
    int pos[V];
    float mu[V];
#pragma unroll
    for (int k = 0; k < V; ++k) {
        pos[k] = s_cnt[rl * C + g * V + k];
        mu[k] = __ldg(means + g * V + k);
    }
    auto put = [&](int r, int k, int x) {
        int at = 0;
        float m = 0.f;
#pragma unroll
        for (int q = 0; q < V; ++q)
            if (q == k) {
                at = pos[q]++;
                m = mu[q];
            }
        if (at < cap) {
            const long long t = (long long)(first_row + r0 + r);
            int4 rec;
            rec.x = (int)(unsigned)(t & 0xffffffffLL);
            rec.y = (int)(t >> 32);
            rec.z = g * V + k;
            rec.w = __float_as_int(__fsub_rn((float)x, m));
            out[at] = rec;
        }
    };
    if (!reread) {
        for (int i = 0; i < kept; ++i) {
            const uint32_t w = __ldg(e + i);
            put(unpack_r(w), unpack_k(w), unpack_x(w));
        }
    } else {
        for (int r = 0; r < nr; ++r) {
            Row<V> v;
            v.load(p + (int64_t)r * C);
#pragma unroll
            for (int k = 0; k < V; ++k)
                if (v.at(k) <= th[k]) put(r, k, v.at(k));
        }
    }
}

// events [0, min(total, cap)) from device memory to host-mapped memory, 16 bytes per thread and
// contiguous per warp (the emit pass scatters its writes; those stay in HBM)
__global__ void __launch_bounds__(256) tc_copy_kernel(const int4* __restrict__ src, const long long* __restrict__ total,
                                                      int64_t cap, int4* __restrict__ dst,
                                                      long long* __restrict__ total_host) {
    const long long t = *total;
    const int64_t n = min((int64_t)t, cap);
    if (blockIdx.x == 0 && threadIdx.x == 0) *total_host = t;
    // four records per thread per round, loads ahead of the stores
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * step < n; i += 4 * step) {
        int4 v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = __ldcs(src + i + j * step);
#pragma unroll
        for (int j = 0; j < 4; ++j) dst[i + j * step] = v[j];
    }
    for (; i < n; i += step) dst[i] = __ldcs(src + i);
}

// ------------------------------------------------------------------------------------------
// host side

struct Error {
    int status;
    std::string msg;
};

#define TC_CUDA(call)                                                                              \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            throw ::lss::tc::Error{LSS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)}; \
    } while (0)

// the largest int16 x whose mean-removed float value passes the reference's double comparison,
// or -32769 when none does; (float)x - mean is monotone in x, so the passing set is a prefix
static int32_t int_threshold(float mean, float median, float thr) {
    const double lim = -1.0 * (double)thr * (double)median;
    auto hit = [&](int x) {
        volatile float y = (float)x - mean;   // one float32 rounding, as the reference's m_fY[j]
        return (double)y <= lim;
    };
    if (!hit(-32768)) return -32769;
    if (hit(32767)) return 32767;
    int lo = -32768, hi = 32767;   // hit(lo), !hit(hi)
    while (hi - lo > 1) {
        const int mid = lo + (hi - lo) / 2;
        if (hit(mid))
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

struct Slot {
    int16_t* h_stage = nullptr;     // pinned copy of a host push
    int16_t* d_stage = nullptr;     // its device copy
    uint32_t* d_ent = nullptr;
    int* d_ucnt = nullptr;
    int* d_ctot = nullptr;
    int* d_tot = nullptr;
    int4* d_ev = nullptr;           // events in device memory (emit pass)
    long long* d_total = nullptr;
    lss_tc_event* h_ev = nullptr;   // host-mapped events (copy pass)
    int4* d_ev_host = nullptr;
    long long* h_total = nullptr;   // host-mapped event count
    long long* d_total_host = nullptr;
    cudaEvent_t done = nullptr;
    cudaEvent_t tev[LSS_TC_N_STAGES + 1] = {};
    int state = 0;                  // 0 free, 1 in flight, 2 events ready
    int64_t n_rows = 0;
    int64_t n = 0, off = 0;         // ready events and how many were read
};

struct Handle {
    int dev = 0;
    int C = 0;
    lss_tc_params prm{};
    cudaStream_t st = nullptr;
    std::vector<int32_t> ithr;
    std::vector<int16_t> thr16;
    std::vector<uint16_t> en16;
    std::vector<float> means;
    int* d_thr = nullptr;
    int16_t* d_thr16 = nullptr;     // thresholds clamped to int16 and the channels that can cross
    uint16_t* d_en16 = nullptr;
    float* d_means = nullptr;
    int64_t ucap = 0, ctacap = 0, cap = 0;
    Slot slots[kSlots];
    std::deque<int> inflight, ready;   // slot indices in push order
    std::vector<lss_tc_event> spill;   // events of slots that had to be reused before a poll read them
    size_t spill_head = 0;
    int next = 0;
    bool overflow = false;
    int64_t launches = 0;
    double stage_ms[LSS_TC_N_STAGES] = {};
    int64_t timed = 0;
    std::string err;

    void init(const lss_tc_params* p, const float* mu, const float* med) {
        if (!p || !mu || !med) throw Error{LSS_ERR_ARG, "lss_tc_open: null argument"};
        if (p->abi_version != LSS_TC_ABI_VERSION) throw Error{LSS_ERR_ARG, "lss_tc_open: abi_version mismatch"};
        prm = *p;
        C = p->n_chan;
        if (C < 1 || C > LSS_TC_MAX_CHANNELS) throw Error{LSS_ERR_ARG, "lss_tc_open: n_chan must be in 1..4096"};
        if (C % 8 != 0 && C > kUnitsPerCta)
            throw Error{LSS_ERR_ARG, "lss_tc_open: n_chan above 512 must be a multiple of 8"};
        if (p->max_rows < 1) throw Error{LSS_ERR_ARG, "lss_tc_open: max_rows must be positive"};
        if (p->max_rows * (int64_t)C >= (1LL << 31))
            throw Error{LSS_ERR_ARG, "lss_tc_open: max_rows * n_chan must stay below 2^31"};
        if (!(p->threshold_std == p->threshold_std)) throw Error{LSS_ERR_ARG, "lss_tc_open: threshold_std is NaN"};
        if (p->event_cap < 0) throw Error{LSS_ERR_ARG, "lss_tc_open: event_cap must not be negative"};
        cap = p->event_cap > 0 ? p->event_cap : std::max<int64_t>(4096, p->max_rows * C / 16);
        means.assign(mu, mu + C);
        ithr.resize(C);
        for (int c = 0; c < C; ++c) ithr[c] = int_threshold(mu[c], med[c], p->threshold_std);
        dev = p->device;
        TC_CUDA(cudaSetDevice(dev));
        TC_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        // scratch for the largest push: at most max(2 x fill + 2G units at the slab length the
        // geometry stops at, the units of max_rows at the longest slab); CTAs follow
        for (int V : {8, 1}) {
            if (V == 8 && C % 8 != 0) continue;
            if (V == 1 && C > kUnitsPerCta) continue;
            const Geometry gm = geometry(C, p->max_rows, V);
            const int64_t small = std::min<int64_t>((p->max_rows + kMinSlab - 1) / kMinSlab * gm.G,
                                                    2 * kFillUnits + 2LL * gm.G);
            const int64_t units = std::max<int64_t>(gm.nslabs * gm.G, small);
            ucap = std::max(ucap, units);
            ctacap = std::max<int64_t>(ctacap, (units / gm.G + gm.R - 1) / gm.R + 1);
        }
        thr16.resize(C);
        en16.resize(C);
        for (int c = 0; c < C; ++c) {
            thr16[c] = (int16_t)std::max(-32768, ithr[c]);
            en16[c] = ithr[c] >= -32768 ? 0xffffu : 0u;
        }
        TC_CUDA(cudaMalloc(&d_thr, sizeof(int) * C));
        TC_CUDA(cudaMalloc(&d_thr16, sizeof(int16_t) * C));
        TC_CUDA(cudaMalloc(&d_en16, sizeof(uint16_t) * C));
        TC_CUDA(cudaMalloc(&d_means, sizeof(float) * C));
        TC_CUDA(cudaMemcpyAsync(d_thr, ithr.data(), sizeof(int) * C, cudaMemcpyHostToDevice, st));
        TC_CUDA(cudaMemcpyAsync(d_thr16, thr16.data(), sizeof(int16_t) * C, cudaMemcpyHostToDevice, st));
        TC_CUDA(cudaMemcpyAsync(d_en16, en16.data(), sizeof(uint16_t) * C, cudaMemcpyHostToDevice, st));
        TC_CUDA(cudaMemcpyAsync(d_means, means.data(), sizeof(float) * C, cudaMemcpyHostToDevice, st));
        for (Slot& s : slots) {
            TC_CUDA(cudaMalloc(&s.d_ent, sizeof(uint32_t) * ucap * kKeep));
            TC_CUDA(cudaMalloc(&s.d_ucnt, sizeof(int) * ucap));
            TC_CUDA(cudaMalloc(&s.d_ctot, sizeof(int) * ctacap * C));
            TC_CUDA(cudaMalloc(&s.d_tot, sizeof(int) * C));
            TC_CUDA(cudaMalloc(&s.d_ev, sizeof(int4) * cap));
            TC_CUDA(cudaMalloc(&s.d_total, sizeof(long long)));
            TC_CUDA(cudaHostAlloc((void**)&s.h_ev, sizeof(lss_tc_event) * cap, cudaHostAllocMapped | cudaHostAllocPortable));
            TC_CUDA(cudaHostGetDevicePointer((void**)&s.d_ev_host, s.h_ev, 0));
            TC_CUDA(cudaHostAlloc((void**)&s.h_total, sizeof(long long), cudaHostAllocMapped | cudaHostAllocPortable));
            TC_CUDA(cudaHostGetDevicePointer((void**)&s.d_total_host, s.h_total, 0));
            TC_CUDA(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
            for (auto& e : s.tev) TC_CUDA(cudaEventCreate(&e));
        }
        TC_CUDA(cudaStreamSynchronize(st));
    }

    void release() {
        if (st) {
            cudaSetDevice(dev);
            cudaStreamSynchronize(st);
        }
        for (Slot& s : slots) {
            cudaFreeHost(s.h_stage);
            cudaFree(s.d_stage);
            cudaFree(s.d_ent);
            cudaFree(s.d_ucnt);
            cudaFree(s.d_ctot);
            cudaFree(s.d_tot);
            cudaFree(s.d_ev);
            cudaFree(s.d_total);
            cudaFreeHost(s.h_ev);
            cudaFreeHost(s.h_total);
            if (s.done) cudaEventDestroy(s.done);
            for (auto& e : s.tev)
                if (e) cudaEventDestroy(e);
        }
        cudaFree(d_thr);
        cudaFree(d_thr16);
        cudaFree(d_en16);
        cudaFree(d_means);
        if (st) cudaStreamDestroy(st);
        st = nullptr;
    }

    // wait for the oldest push in flight; its events become readable in place
    void collect_oldest() {
        const int i = inflight.front();
        Slot& s = slots[i];
        TC_CUDA(cudaEventSynchronize(s.done));
        inflight.pop_front();
        const long long total = *s.h_total;
        s.n = std::min<int64_t>(total, cap);
        s.off = 0;
        if (total > cap) overflow = true;
        s.state = 2;
        ready.push_back(i);
        if (prm.profile && s.n_rows > 0) {
            for (int k = 0; k < LSS_TC_N_STAGES; ++k) {
                float ms = 0.f;
                TC_CUDA(cudaEventElapsedTime(&ms, s.tev[k], s.tev[k + 1]));
                stage_ms[k] += ms;
            }
            ++timed;
        }
    }

    // the oldest ready slot's unread events move to the spill queue and the slot is free again
    void spill_oldest() {
        const int i = ready.front();
        Slot& s = slots[i];
        if (spill_head > 0 && spill_head * 2 >= spill.size()) {
            spill.erase(spill.begin(), spill.begin() + (ptrdiff_t)spill_head);
            spill_head = 0;
        }
        spill.insert(spill.end(), s.h_ev + s.off, s.h_ev + s.n);
        ready.pop_front();
        s.state = 0;
    }

    Slot& free_slot() {
        for (;;) {
            for (int k = 0; k < kSlots; ++k) {
                const int i = (next + k) % kSlots;
                if (slots[i].state == 0) {
                    next = (i + 1) % kSlots;
                    return slots[i];
                }
            }
            if (ready.empty()) collect_oldest();
            spill_oldest();
        }
    }

    int64_t available() const {
        int64_t n = (int64_t)(spill.size() - spill_head);
        for (int i : ready) n += slots[i].n - slots[i].off;
        return n;
    }

    int64_t read(lss_tc_event* out, int64_t cap_out) {
        int64_t got = 0;
        if (spill_head < spill.size()) {
            const int64_t k = std::min<int64_t>(cap_out, (int64_t)(spill.size() - spill_head));
            par_memcpy(out, spill.data() + spill_head, sizeof(lss_tc_event) * (size_t)k);
            spill_head += (size_t)k;
            got += k;
        }
        while (got < cap_out && !ready.empty()) {
            Slot& s = slots[ready.front()];
            const int64_t k = std::min(cap_out - got, s.n - s.off);
            if (k > 0) par_memcpy(out + got, s.h_ev + s.off, sizeof(lss_tc_event) * (size_t)k);
            s.off += k;
            got += k;
            if (s.off == s.n) {
                s.state = 0;
                ready.pop_front();
            }
        }
        return got;
    }

    void launch(Slot& s, const int16_t* d_rows, int64_t n_rows, int64_t first_row) {
        const int V = (C % 8 == 0 && (reinterpret_cast<uintptr_t>(d_rows) & 15) == 0) ? 8 : 1;
        if (V == 1 && C > kUnitsPerCta)
            throw Error{LSS_ERR_ARG, "device rows must be 16-byte aligned for n_chan above 512"};
        const Geometry gm = geometry(C, n_rows, V);
        if (gm.nslabs * gm.G > ucap || gm.nctas > ctacap) throw Error{LSS_ERR_INTERNAL, "scratch too small"};
        const int threads = gm.R * gm.G;
        const size_t sm_slabs = sizeof(int) * (size_t)gm.R * C;
        const size_t sm_emit = sm_slabs + sizeof(int) * C;
        if (V == 8) {
            tc_count8_kernel<<<(unsigned)gm.nctas, threads, sizeof(int) * C, st>>>(
                d_rows, n_rows, C, gm.G, gm.S, gm.R, gm.nslabs, d_thr16, d_en16, s.d_ent, s.d_ucnt, s.d_ctot);
        } else {
            tc_count1_kernel<<<(unsigned)gm.nctas, threads, sm_slabs, st>>>(
                d_rows, n_rows, C, gm.G, gm.S, gm.R, gm.nslabs, d_thr, s.d_ent, s.d_ucnt, s.d_ctot);
        }
        TC_CUDA(cudaGetLastError());
        if (prm.profile) TC_CUDA(cudaEventRecord(s.tev[2], st));
        tc_offsets_kernel<<<(C + 31) / 32, 1024, 0, st>>>(s.d_ctot, gm.nctas, C, s.d_tot);
        TC_CUDA(cudaGetLastError());
        if (prm.profile) TC_CUDA(cudaEventRecord(s.tev[3], st));
        if (V == 8) {
            tc_emit_kernel<8><<<(unsigned)gm.nctas, threads, sm_emit, st>>>(
                d_rows, n_rows, C, gm.G, gm.S, gm.R, gm.nslabs, d_thr, d_means, s.d_ent, s.d_ucnt, s.d_ctot,
                s.d_tot, first_row, s.d_ev, cap, s.d_total);
        } else {
            tc_emit_kernel<1><<<(unsigned)gm.nctas, threads, sm_emit, st>>>(
                d_rows, n_rows, C, gm.G, gm.S, gm.R, gm.nslabs, d_thr, d_means, s.d_ent, s.d_ucnt, s.d_ctot,
                s.d_tot, first_row, s.d_ev, cap, s.d_total);
        }
        TC_CUDA(cudaGetLastError());
        if (prm.profile) TC_CUDA(cudaEventRecord(s.tev[4], st));
        const int64_t most = std::min<int64_t>(cap, n_rows * C);
        const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(152 * 8, (most + 255) / 256));
        tc_copy_kernel<<<blocks, 256, 0, st>>>(s.d_ev, s.d_total, cap, s.d_ev_host, s.d_total_host);
        TC_CUDA(cudaGetLastError());
        launches = 4;
    }

    void push(const int16_t* rows, int64_t n_rows, int64_t first_row, bool device) {
        if (n_rows < 0 || n_rows > prm.max_rows) throw Error{LSS_ERR_ARG, "n_rows must be in 0..max_rows"};
        if (n_rows > 0 && !rows) throw Error{LSS_ERR_ARG, "null rows"};
        TC_CUDA(cudaSetDevice(dev));
        Slot& s = free_slot();
        s.n_rows = n_rows;
        launches = 0;
        if (prm.profile) TC_CUDA(cudaEventRecord(s.tev[0], st));
        const int16_t* d_rows = rows;
        if (n_rows > 0 && !device) {
            if (!s.h_stage) {
                TC_CUDA(cudaHostAlloc((void**)&s.h_stage, sizeof(int16_t) * prm.max_rows * C, cudaHostAllocPortable));
                TC_CUDA(cudaMalloc(&s.d_stage, sizeof(int16_t) * prm.max_rows * C));
            }
            const size_t bytes = sizeof(int16_t) * (size_t)n_rows * C;
            par_memcpy(s.h_stage, rows, bytes);
            TC_CUDA(cudaMemcpyAsync(s.d_stage, s.h_stage, bytes, cudaMemcpyHostToDevice, st));
            d_rows = s.d_stage;
        }
        if (prm.profile) TC_CUDA(cudaEventRecord(s.tev[1], st));
        if (n_rows > 0) {
            launch(s, d_rows, n_rows, first_row);
        } else {
            *s.h_total = 0;   // no kernel of this slot is in flight
            if (prm.profile)
                for (int k = 2; k < LSS_TC_N_STAGES; ++k) TC_CUDA(cudaEventRecord(s.tev[k], st));
        }
        if (prm.profile) TC_CUDA(cudaEventRecord(s.tev[LSS_TC_N_STAGES], st));
        TC_CUDA(cudaEventRecord(s.done, st));
        s.state = 1;
        inflight.push_back((int)(&s - slots));
    }
};

}  // namespace tc
}  // namespace lss

struct lss_tc_handle {
    lss::tc::Handle h;
};

#define TC_TRY(hp, ...)                                                                            \
    try {                                                                                          \
        __VA_ARGS__;                                                                               \
        return LSS_OK;                                                                             \
    } catch (const lss::tc::Error& e) {                                                            \
        (hp)->h.err = e.msg;                                                                       \
        return e.status;                                                                           \
    } catch (const std::bad_alloc&) {                                                              \
        (hp)->h.err = "host allocation failed";                                                    \
        return LSS_ERR_NOMEM;                                                                      \
    } catch (const std::exception& e) {                                                            \
        (hp)->h.err = e.what();                                                                    \
        return LSS_ERR_INTERNAL;                                                                   \
    }

extern "C" {

int lss_tc_default_params(lss_tc_params* p) {
    if (!p) return LSS_ERR_ARG;
    std::memset(p, 0, sizeof(*p));
    p->abi_version = LSS_TC_ABI_VERSION;
    p->device = 0;
    p->n_chan = 0;
    p->threshold_std = 3.f;
    p->max_rows = 1500;
    p->event_cap = 0;
    p->profile = 0;
    return LSS_OK;
}

int lss_tc_int_thresholds(int32_t n_chan, const float* means, const float* medians, float threshold_std,
                          int32_t* out) {
    if (n_chan < 0 || (n_chan > 0 && (!means || !medians || !out))) {
        lss::g_handleless_error = "lss_tc_int_thresholds: bad argument";
        return LSS_ERR_ARG;
    }
    for (int c = 0; c < n_chan; ++c) out[c] = lss::tc::int_threshold(means[c], medians[c], threshold_std);
    return LSS_OK;
}

int lss_tc_calibrate(const int16_t* rows, int64_t n_rows, int32_t n_chan, float* means, float* medians) {
    if (!rows || n_rows < 1 || n_chan < 1 || !means || !medians) {
        lss::g_handleless_error = "lss_tc_calibrate: bad argument";
        return LSS_ERR_ARG;
    }
    try {
        std::vector<float> col((size_t)n_rows);
        for (int c = 0; c < n_chan; ++c) {
            int64_t sum = 0;
            for (int64_t j = 0; j < n_rows; ++j) sum += rows[j * n_chan + c];
            const float mu = (float)sum / (float)n_rows;
            for (int64_t j = 0; j < n_rows; ++j) {
                volatile float y = (float)rows[j * n_chan + c] - mu;
                col[(size_t)j] = std::fabs((float)y);
            }
            std::nth_element(col.begin(), col.begin() + n_rows / 2, col.end());
            means[c] = mu;
            medians[c] = col[(size_t)(n_rows / 2)];
        }
    } catch (const std::bad_alloc&) {
        lss::g_handleless_error = "lss_tc_calibrate: host allocation failed";
        return LSS_ERR_NOMEM;
    }
    return LSS_OK;
}

int lss_tc_open(const lss_tc_params* p, const float* means, const float* medians, lss_tc_handle** out) {
    if (!out) return LSS_ERR_ARG;
    *out = nullptr;
    lss_tc_handle* h = nullptr;
    try {
        h = new lss_tc_handle();
        h->h.init(p, means, medians);
        *out = h;
        return LSS_OK;
    } catch (const lss::tc::Error& e) {
        lss::g_handleless_error = e.msg;
        if (h) h->h.release();
        delete h;
        return e.status;
    } catch (const std::exception& e) {
        lss::g_handleless_error = e.what();
        if (h) h->h.release();
        delete h;
        return LSS_ERR_INTERNAL;
    }
}

int lss_tc_push(lss_tc_handle* hp, const int16_t* rows, int64_t n_rows, int64_t first_row_sample) {
    if (!hp) return LSS_ERR_ARG;
    TC_TRY(hp, hp->h.push(rows, n_rows, first_row_sample, false));
}

int lss_tc_push_device(lss_tc_handle* hp, const int16_t* dev_rows, int64_t n_rows, int64_t first_row_sample) {
    if (!hp) return LSS_ERR_ARG;
    TC_TRY(hp, hp->h.push(dev_rows, n_rows, first_row_sample, true));
}

int lss_tc_poll(lss_tc_handle* hp, lss_tc_event* out, int64_t cap, int64_t* n_out) {
    if (!hp || !n_out || cap < 0 || (cap > 0 && !out)) return LSS_ERR_ARG;
    *n_out = 0;
    lss::tc::Handle& h = hp->h;
    try {
        TC_CUDA(cudaSetDevice(h.dev));
        while (h.available() == 0 && !h.inflight.empty()) h.collect_oldest();
        *n_out = h.read(out, cap);
        if (h.overflow) {
            h.overflow = false;
            h.err = "event buffer overflow: events beyond event_cap of a push were dropped";
            return LSS_ERR_OVERFLOW;
        }
        return LSS_OK;
    } catch (const lss::tc::Error& e) {
        h.err = e.msg;
        return e.status;
    } catch (const std::exception& e) {
        h.err = e.what();
        return LSS_ERR_INTERNAL;
    }
}

int lss_tc_pending(lss_tc_handle* hp, int64_t* n) {
    if (!hp || !n) return LSS_ERR_ARG;
    TC_TRY(hp, {
        TC_CUDA(cudaSetDevice(hp->h.dev));
        while (!hp->h.inflight.empty()) hp->h.collect_oldest();
        *n = hp->h.available();
    });
}

int lss_tc_thresholds(const lss_tc_handle* hp, int32_t* out, int32_t n) {
    if (!hp || !out || n != hp->h.C) return LSS_ERR_ARG;
    std::memcpy(out, hp->h.ithr.data(), sizeof(int32_t) * (size_t)n);
    return LSS_OK;
}

int lss_tc_cuda_stream(const lss_tc_handle* hp, void** stream) {
    if (!hp || !stream) return LSS_ERR_ARG;
    *stream = (void*)hp->h.st;
    return LSS_OK;
}

int lss_tc_kernel_launches(const lss_tc_handle* hp, int64_t* n) {
    if (!hp || !n) return LSS_ERR_ARG;
    *n = hp->h.launches;
    return LSS_OK;
}

int lss_tc_stage_times(lss_tc_handle* hp, double* ms, int32_t n, int64_t* n_pushes) {
    if (!hp || !ms || n < LSS_TC_N_STAGES) return LSS_ERR_ARG;
    TC_TRY(hp, {
        TC_CUDA(cudaSetDevice(hp->h.dev));
        while (!hp->h.inflight.empty()) hp->h.collect_oldest();
        for (int k = 0; k < LSS_TC_N_STAGES; ++k) ms[k] = hp->h.stage_ms[k];
        if (n_pushes) *n_pushes = hp->h.timed;
    });
}

int lss_tc_close(lss_tc_handle* hp) {
    if (!hp) return LSS_ERR_ARG;
    hp->h.release();
    delete hp;
    return LSS_OK;
}

const char* lss_tc_last_error(const lss_tc_handle* hp) {
    return hp ? hp->h.err.c_str() : lss::g_handleless_error.c_str();
}

}  // extern "C"
