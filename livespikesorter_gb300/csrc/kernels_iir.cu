// kernels_iir.cu -- the stateful high-pass mode: a causal Butterworth high-pass as a cascade of
// second-order sections (direct form II transposed, FP32 state per channel) run over the stream
// once, with the state carried from batch to batch on the device, followed by the median common
// average reference.  It replaces Kilosort's circular zero-phase filter (preprocessing.py:120-136,
// OnlineSpikesV2.cu:1006-1056), whose result depends on each whole batch window; the filter itself
// is the one Kilosort designs there (scipy butter(3, 300 Hz, 'high')), applied forward only.
//
// The recurrence is sequential in time, so the rows of a group are cut into chunks of kIirChunk
// rows and solved in three passes:
//   1. zero-state pass: per (chunk, channel), the cascade's state at the chunk's end when it
//      starts from zero;
//   2. scan: per channel, sequentially over the chunks, the state entering each chunk,
//      s[k+1] = P s[k] + z[k] with P = A^kIirChunk the state transition over a whole chunk;
//   3. apply: per chunk, the cascade run again from its entering state over the chunk's rows (each
//      row of every channel into shared memory), then per row the lower median across channels is
//      subtracted and the row is written to every window that holds it, in the whitening GEMM's
//      operand format.
// A chain is a run of rows filtered continuously: the whole group on the streaming path (its state
// enters from the previous group, or is the steady state of the first row at a segment start), or
// each window alone on the windows API.
#include "lss_kernels.cuh"
#include "lss_select.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

namespace lss {

// ----------------------------------------------------------------------------------------------
// design (host, double): Butterworth high-pass of the given order as second-order sections
// ----------------------------------------------------------------------------------------------
// The analog low-pass prototype's poles exp(i pi (2k + N + 1) / 2N) are mapped to a high-pass of
// the pre-warped edge w = 2 fs tan(pi fc / fs) (s -> w / s, zeros at s = 0), then to the z plane by
// the bilinear transform z = (2 fs + s) / (2 fs - s), zeros at z = 1.  Sections: each complex pole
// pair with two zeros at 1, a real pole with one; ordered by pole radius (the pole nearest the unit
// circle last) and the overall gain, fixed so that |H(-1)| = 1, on the first section.  Each section
// is (b0, b1, b2, 1, a1, a2).
int butter_highpass_sos(int order, double fc, double fs, std::vector<double>& sos) {
    if (order < 1 || order > 2 * kIirMaxSections || !(fs > 0.0) || !(fc > 0.0) || !(fc < fs / 2)) return -1;
    const double pi = 3.14159265358979323846;
    const double w = 2.0 * fs * std::tan(pi * fc / fs);
    std::vector<std::complex<double>> zp;   // digital poles
    for (int k = 0; k < order; ++k) {
        const std::complex<double> p = std::polar(1.0, pi * (2.0 * k + order + 1) / (2.0 * order));
        const std::complex<double> s = w / p;
        zp.push_back((2.0 * fs + s) / (2.0 * fs - s));
    }
    struct Sec {
        double r;   // pole radius (ordering)
        double b[3], a[3];
    };
    std::vector<Sec> secs;
    std::vector<bool> used(zp.size(), false);
    for (size_t i = 0; i < zp.size(); ++i) {
        if (used[i]) continue;
        used[i] = true;
        const std::complex<double> p = zp[i];
        Sec sc{};
        if (std::fabs(p.imag()) > 1e-12 * std::abs(p)) {
            for (size_t j = i + 1; j < zp.size(); ++j)   // its conjugate
                if (!used[j] && std::abs(zp[j] - std::conj(p)) < 1e-9) {
                    used[j] = true;
                    break;
                }
            sc.b[0] = 1.0, sc.b[1] = -2.0, sc.b[2] = 1.0;
            sc.a[0] = 1.0, sc.a[1] = -2.0 * p.real(), sc.a[2] = std::norm(p);
        } else {
            sc.b[0] = 1.0, sc.b[1] = -1.0, sc.b[2] = 0.0;
            sc.a[0] = 1.0, sc.a[1] = -p.real(), sc.a[2] = 0.0;
        }
        sc.r = std::abs(p);
        secs.push_back(sc);
    }
    std::stable_sort(secs.begin(), secs.end(), [](const Sec& x, const Sec& y) { return x.r < y.r; });
    // gain: |H(z = -1)| = 1 at the Nyquist frequency
    std::complex<double> h = 1.0;
    const std::complex<double> zm1 = -1.0;
    for (const Sec& sc : secs)
        h *= (sc.b[0] + sc.b[1] / zm1 + sc.b[2] / (zm1 * zm1)) / (sc.a[0] + sc.a[1] / zm1 + sc.a[2] / (zm1 * zm1));
    const double g = 1.0 / std::abs(h);
    for (int j = 0; j < 3; ++j) secs[0].b[j] *= g;
    sos.clear();
    for (const Sec& sc : secs)
        for (double v : {sc.b[0], sc.b[1], sc.b[2], sc.a[0], sc.a[1], sc.a[2]}) sos.push_back(v);
    return (int)secs.size();
}

// one step of the cascade in double (host): state z [2 per section], input x -> output
static double cascade_step(const std::vector<double>& sos, int ns, double* z, double x) {
    double u = x;
    for (int s = 0; s < ns; ++s) {
        const double* c = &sos[6 * s];
        const double y = c[0] * u + z[2 * s];
        z[2 * s] = c[1] * u - c[4] * y + z[2 * s + 1];
        z[2 * s + 1] = c[2] * u - c[5] * y;
        u = y;
    }
    return u;
}

IirCoeffs make_iir_coeffs(const std::vector<double>& sos, std::vector<float>& powers) {
    const int ns = (int)(sos.size() / 6);
    IirCoeffs k{};
    k.ns = kIirMaxSections;
    for (int s = 0; s < kIirMaxSections; ++s) {
        if (s < ns) {
            const double* c = &sos[6 * s];
            k.b[s][0] = (float)c[0], k.b[s][1] = (float)c[1], k.b[s][2] = (float)c[2];
            k.a[s][0] = (float)c[4], k.a[s][1] = (float)c[5];
        } else {   // identity section
            k.b[s][0] = 1.f;
        }
    }
    // steady state of a unit constant input: per section z1 = y - b0 u, z2 = b2 u - a2 y with
    // y = H_s(1) u, the next section's input being y (sosfilt_zi's construction)
    double u = 1.0;
    for (int s = 0; s < kIirMaxSections; ++s) {
        double c[6] = {1, 0, 0, 1, 0, 0};
        if (s < ns) std::copy(&sos[6 * s], &sos[6 * s] + 6, c);
        const double y = (c[0] + c[1] + c[2]) / (1.0 + c[4] + c[5]) * u;
        k.zi[2 * s] = (float)(y - c[0] * u);
        k.zi[2 * s + 1] = (float)(c[2] * u - c[5] * y);
        u = y;
    }
    // A: the state transition with zero input (column j = one step from unit state j); P = A^chunk
    std::vector<double> pad(sos);
    for (int s = ns; s < kIirMaxSections; ++s)
        for (double v : {1.0, 0.0, 0.0, 1.0, 0.0, 0.0}) pad.push_back(v);
    constexpr int S = 2 * kIirMaxSections;
    double A[S][S], P[S][S];
    for (int j = 0; j < S; ++j) {
        double z[S] = {};
        z[j] = 1.0;
        cascade_step(pad, kIirMaxSections, z, 0.0);
        for (int i = 0; i < S; ++i) A[i][j] = z[i];
    }
    for (int i = 0; i < S; ++i)
        for (int j = 0; j < S; ++j) P[i][j] = i == j;
    for (int n = 0; n < kIirChunk; ++n) {
        double Q[S][S];
        for (int i = 0; i < S; ++i)
            for (int j = 0; j < S; ++j) {
                double acc = 0.0;
                for (int q = 0; q < S; ++q) acc += A[i][q] * P[q][j];
                Q[i][j] = acc;
            }
        std::copy(&Q[0][0], &Q[0][0] + S * S, &P[0][0]);
    }
    for (int i = 0; i < S; ++i)
        for (int j = 0; j < S; ++j) k.P[i * S + j] = (float)P[i][j];
    // P^0 .. P^kIirChunk for the warp scan
    powers.assign((size_t)(kIirChunk + 1) * S * S, 0.f);
    double Q[S][S];
    for (int i = 0; i < S; ++i)
        for (int j = 0; j < S; ++j) Q[i][j] = i == j;
    for (int n = 0; n <= kIirChunk; ++n) {
        for (int i = 0; i < S; ++i)
            for (int j = 0; j < S; ++j) powers[(size_t)n * S * S + i * S + j] = (float)Q[i][j];
        double R[S][S];
        for (int i = 0; i < S; ++i)
            for (int j = 0; j < S; ++j) {
                double acc = 0.0;
                for (int q = 0; q < S; ++q) acc += P[i][q] * Q[q][j];
                R[i][j] = acc;
            }
        std::copy(&R[0][0], &R[0][0] + S * S, &Q[0][0]);
    }
    return k;
}

// ----------------------------------------------------------------------------------------------
// device
// ----------------------------------------------------------------------------------------------
static_assert(kIirMaxSections == 2, "the kernels hold the cascade state in one float4");

__device__ __forceinline__ float iir_step(const IirCoeffs& k, float4& z, float x) {
    float u = x;
    float y = fmaf(k.b[0][0], u, z.x);
    z.x = fmaf(-k.a[0][0], y, fmaf(k.b[0][1], u, z.y));
    z.y = fmaf(-k.a[0][1], y, k.b[0][2] * u);
    u = y;
    y = fmaf(k.b[1][0], u, z.z);
    z.z = fmaf(-k.a[1][0], y, fmaf(k.b[1][1], u, z.w));
    z.w = fmaf(-k.a[1][1], y, k.b[1][2] * u);
    return y;
}

// rows of chunk q: [r0, r1) of the group's rows, and whether it starts a chain
struct ChunkRows {
    int r0, r1;
    bool first;
    int chain;
};
__device__ __forceinline__ ChunkRows chunk_rows(int q, const IirGroup& g) {
    ChunkRows c;
    if (g.independent) {
        const int cpw = (g.W + kIirChunk - 1) / kIirChunk;
        const int b = q / cpw, i = q - b * cpw;
        c.r0 = b * g.NT + i * kIirChunk;
        c.r1 = b * g.NT + min(g.W, (i + 1) * kIirChunk);
        c.first = i == 0;
        c.chain = b;
    } else {
        c.r0 = q * kIirChunk;
        c.r1 = min(g.span, c.r0 + kIirChunk);
        c.first = q == 0;
        c.chain = 0;
    }
    return c;
}

constexpr int kIirThreads = 128;

__global__ void __launch_bounds__(kIirThreads)
iir_zero_state_kernel(const int16_t* __restrict__ raw, int64_t row_stride, const int32_t* __restrict__ chan, int C,
                      IirGroup g, IirCoeffs k, float4* __restrict__ zs) {
    const int q = blockIdx.x;
    const int c = blockIdx.y * kIirThreads + threadIdx.x;
    if (c >= C) return;
    const ChunkRows cr = chunk_rows(q, g);
    const int src = chan ? chan[c] : c;
    float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int r = cr.r0; r < cr.r1; ++r) iir_step(k, z, (float)raw[(int64_t)r * row_stride + src]);
    zs[(int64_t)q * C + c] = z;
}

__device__ __forceinline__ float4 matvec4(const float* P, const float4 s, const float4 add) {
    float4 n;
    n.x = fmaf(P[0], s.x, fmaf(P[1], s.y, fmaf(P[2], s.z, fmaf(P[3], s.w, add.x))));
    n.y = fmaf(P[4], s.x, fmaf(P[5], s.y, fmaf(P[6], s.z, fmaf(P[7], s.w, add.y))));
    n.z = fmaf(P[8], s.x, fmaf(P[9], s.y, fmaf(P[10], s.z, fmaf(P[11], s.w, add.z))));
    n.w = fmaf(P[12], s.x, fmaf(P[13], s.y, fmaf(P[14], s.z, fmaf(P[15], s.w, add.w))));
    return n;
}

__device__ __forceinline__ float4 shfl_up4(float4 v, int d) {
    return make_float4(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d),
                       __shfl_up_sync(0xffffffffu, v.z, d), __shfl_up_sync(0xffffffffu, v.w, d));
}

constexpr int kScanWarps = 4;

// Streaming chain: one warp per channel, 32 chunks per step.  With the same transition P for every
// chunk, the end state of chunk i when chunk q0 is entered with zero state is the prefix
// v_i = sum_{j <= i} P^(i-j) z_j, a warp scan (v_i += P^d v_(i-d) for d = 1, 2, 4, 8, 16); the state
// entering chunk q0 + i is P^i s0 + v_(i-1), and s0 advances to P^32 s0 + v_31.  pw = P^0 .. P^32.
__global__ void __launch_bounds__(kScanWarps * 32)
iir_scan_stream_kernel(const int16_t* __restrict__ raw, int64_t row_stride, const int32_t* __restrict__ chan, int C,
                       IirGroup g, IirCoeffs k, const float* __restrict__ pw, const float4* __restrict__ zs,
                       const float4* __restrict__ carried, float4* __restrict__ sin) {
    __shared__ float s_pw[(kIirChunk + 1) * 16];
    for (int i = threadIdx.x; i < (kIirChunk + 1) * 16; i += blockDim.x) s_pw[i] = pw[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * kScanWarps + (threadIdx.x >> 5);
    if (c >= C) return;
    float4 s0;
    if (g.reset) {
        const float x0 = (float)raw[chan ? chan[c] : c];
        s0 = make_float4(k.zi[0] * x0, k.zi[1] * x0, k.zi[2] * x0, k.zi[3] * x0);
    } else {
        s0 = carried[c];
    }
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int q0 = 0; q0 < g.chunks; q0 += 32) {
        const int q = q0 + lane;
        float4 v = q < g.chunks ? zs[(int64_t)q * C + c] : z4;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const float4 t = shfl_up4(v, d);
            if (lane >= d) v = matvec4(s_pw + d * 16, t, v);
        }
        float4 ev = shfl_up4(v, 1);
        if (lane == 0) ev = z4;
        if (q < g.chunks) sin[(int64_t)q * C + c] = matvec4(s_pw + lane * 16, s0, ev);
        const float4 v31 = make_float4(__shfl_sync(0xffffffffu, v.x, 31), __shfl_sync(0xffffffffu, v.y, 31),
                                       __shfl_sync(0xffffffffu, v.z, 31), __shfl_sync(0xffffffffu, v.w, 31));
        s0 = matvec4(s_pw + 32 * 16, s0, v31);
    }
}

// Windows API: every window its own chain, one thread per (window, channel), sequentially over the
// window's chunks from the steady state of its first row
__global__ void __launch_bounds__(kIirThreads)
iir_scan_windows_kernel(const int16_t* __restrict__ raw, int64_t row_stride, const int32_t* __restrict__ chan, int C,
                        IirGroup g, IirCoeffs k, const float* __restrict__ pw, const float4* __restrict__ zs,
                        float4* __restrict__ sin) {
    const int c = blockIdx.x * kIirThreads + threadIdx.x;
    const int b = blockIdx.y;
    if (c >= C) return;
    const int cpw = (g.W + kIirChunk - 1) / kIirChunk;
    const float x0 = (float)raw[(int64_t)b * g.NT * row_stride + (chan ? chan[c] : c)];
    float4 s = make_float4(k.zi[0] * x0, k.zi[1] * x0, k.zi[2] * x0, k.zi[3] * x0);
    for (int i = 0; i < cpw; ++i) {
        const int64_t q = (int64_t)b * cpw + i;
        sin[q * C + c] = s;
        s = matvec4(pw + 16, s, zs[q * C + c]);
    }
}

constexpr int kIirApplyThreads = 256;

// OUT: 0 = FP32, 1 = TF32 split (Y = tf32(y), Ylo = y - Y when Ylo is given), 2 = BF16 split (Y /
// Ylo viewed as bf16)
template <int NJ, int OUT>
__global__ void __launch_bounds__(kIirApplyThreads)
iir_apply_car_kernel(const int16_t* __restrict__ raw, int64_t row_stride, const int32_t* __restrict__ chan, int C,
                     IirGroup g, IirCoeffs k, const float4* __restrict__ sin, float4* __restrict__ carried,
                     float* __restrict__ Y, float* __restrict__ Ylo) {
    extern __shared__ float s_y[];   // [kIirChunk][C + 1]
    const int q = blockIdx.x;
    const ChunkRows cr = chunk_rows(q, g);
    const int ld = C + 1;
    for (int c = threadIdx.x; c < C; c += kIirApplyThreads) {
        const int src = chan ? chan[c] : c;
        float4 z = sin[(int64_t)q * C + c];
#pragma unroll 8
        for (int r = cr.r0; r < cr.r1; ++r) {
            // the state entering the next group's first row (streaming chains only)
            if (!g.independent && r == g.carry_row) carried[c] = z;
            s_y[(r - cr.r0) * ld + c] = iir_step(k, z, (float)raw[(int64_t)r * row_stride + src]);
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int rr = warp; rr < cr.r1 - cr.r0; rr += kIirApplyThreads / 32) {
        float v[NJ];
        uint32_t key[NJ];
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            const int c = lane + 32 * j;
            v[j] = c < C ? s_y[rr * ld + c] : 0.f;
            key[j] = c < C ? float_key(v[j]) : 0xffffffffu;
        }
        const float med = key_float(warp_kth_smallest<NJ>(key, (C - 1) >> 1));
        const int r = cr.r0 + rr;
        // the windows holding row r: b with 0 <= r - b NT < W (one, on the windows API)
        int b_lo, b_hi;
        if (g.independent) {
            b_lo = b_hi = cr.chain;
        } else {
            b_hi = min(g.nb - 1, r / g.NT);
            b_lo = r >= g.W ? (r - g.W) / g.NT + 1 : 0;
        }
        for (int b = b_lo; b <= b_hi; ++b) {
            const int64_t o = ((int64_t)b * g.W + (r - b * g.NT)) * C;
#pragma unroll
            for (int j = 0; j < NJ; ++j) {
                const int c = lane + 32 * j;
                if (c >= C) continue;
                const float y = v[j] - med;
                if constexpr (OUT == 2) {
                    const __nv_bfloat16 h = __float2bfloat16_rn(y);
                    reinterpret_cast<__nv_bfloat16*>(Y)[o + c] = h;
                    reinterpret_cast<__nv_bfloat16*>(Ylo)[o + c] = __float2bfloat16_rn(y - __bfloat162float(h));
                } else if constexpr (OUT == 1) {
                    uint32_t h;
                    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(y));
                    Y[o + c] = __uint_as_float(h);
                    if (Ylo) Ylo[o + c] = y - __uint_as_float(h);
                } else {
                    Y[o + c] = y;
                }
            }
        }
    }
}

int iir_chunks(const IirGroup& g) {
    return g.independent ? g.nb * ((g.W + kIirChunk - 1) / kIirChunk) : (g.span + kIirChunk - 1) / kIirChunk;
}

cudaError_t launch_iir_car(const int16_t* raw, int64_t row_stride, const int32_t* chan, int C, IirGroup g,
                           const IirCoeffs& k, const float* pw, float4* zs, float4* sin, float4* carried, float* Y,
                           float* Ylo, int out_mode, cudaStream_t s, int64_t& nl) {
    g.chunks = iir_chunks(g);
    if (g.chunks <= 0 || C <= 0 || C > 1024 || (out_mode == 2 && !Ylo)) return cudaErrorInvalidValue;
    const dim3 g1(g.chunks, (C + kIirThreads - 1) / kIirThreads);
    iir_zero_state_kernel<<<g1, kIirThreads, 0, s>>>(raw, row_stride, chan, C, g, k, zs);
    if (g.independent)
        iir_scan_windows_kernel<<<dim3((C + kIirThreads - 1) / kIirThreads, g.nb), kIirThreads, 0, s>>>(
            raw, row_stride, chan, C, g, k, pw, zs, sin);
    else
        iir_scan_stream_kernel<<<(C + kScanWarps - 1) / kScanWarps, kScanWarps * 32, 0, s>>>(raw, row_stride, chan, C,
                                                                                          g, k, pw, zs, carried, sin);
    const size_t smem = (size_t)kIirChunk * (C + 1) * sizeof(float);
    const int nj = (C + 31) / 32;
    cudaError_t e = cudaSuccess;
#define LSS_IIR(N, O)                                                                                         \
    do {                                                                                                      \
        e = raise_smem_limit((const void*)iir_apply_car_kernel<N, O>, smem);                                  \
        if (e == cudaSuccess)                                                                                 \
            iir_apply_car_kernel<N, O><<<g.chunks, kIirApplyThreads, smem, s>>>(raw, row_stride, chan, C, g, k, \
                                                                               sin, carried, Y, Ylo);         \
    } while (0)
#define LSS_IIR_NJ(N)               \
    do {                            \
        if (out_mode == 2)          \
            LSS_IIR(N, 2);          \
        else if (out_mode == 1)     \
            LSS_IIR(N, 1);          \
        else                        \
            LSS_IIR(N, 0);          \
    } while (0)
    if (nj <= 4) LSS_IIR_NJ(4);
    else if (nj <= 8) LSS_IIR_NJ(8);
    else if (nj <= 12) LSS_IIR_NJ(12);
    else if (nj <= 16) LSS_IIR_NJ(16);
    else LSS_IIR_NJ(32);
#undef LSS_IIR_NJ
#undef LSS_IIR
    nl += 3;
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace lss
