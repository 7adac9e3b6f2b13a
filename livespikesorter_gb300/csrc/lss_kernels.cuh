// lss_kernels.cuh -- device kernels of the per-batch sorting path and their launchers.
//
// Data layout in HBM (time-major everywhere, so every stage reads and writes rows that are
// contiguous across channels or templates):
//   raw      int16 [S][Cin]            one contiguous span; window b starts at row b*NT
//   Xw       f32   [nb][W+L+R][C]      median-CAR'd window, circularly wrapped by L/R rows
//   Y        f32   [nb][W][C]          high-passed
//   Z        f32   [nb][W][C]          whitened + drift-corrected (M @ Wrot); becomes Xres
//   Bpc      f32   [nb][W][K][C]       temporal-basis convolution
//   Bt       f32   [nb][W][T]          template scores B transposed (templates contiguous)
//   ctcP     f32   [T][2nt+1][T]       ctcP[s][l][t] = ctc[t][s][l]  (target template contiguous)
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <vector>

namespace lss {

// Per-batch results of the matching loop (device).
struct MatchOut {
    int* n_spikes;     // [nb] spikes accepted (may exceed cap: then the list is truncated)
    int* n_iters;      // [nb] iterations that accepted spikes
    int* status;       // [nb] bit 0 = spike list overflow, bit 1 = bad launch shape
    int* sp_w;         // [nb][cap] window sample
    int* sp_t;         // [nb][cap] template
    float* sp_amp;     // [nb][cap]
    int* sp_iter;      // [nb][cap]
    int cap;
};

// Exact re-score of accepted candidates when the scores come from a low-precision projection
// (bt0 null: off).  An accepted (t, w) takes the amplitude (B[w][t] + exact - bt0[w][t]) / nm[t]:
// its running score corrected by the difference between the FP32 projection of the exact operands,
// sum_i wall3[t][i] (x_hi[w][i] + x_lo[w][i]), and the low-precision initial score bt0.
struct MatchRescore {
    const float* bt0 = nullptr;       // [nb][W][T] the initial low-precision scores
    const uint16_t* x_hi = nullptr;   // [nb][W][kc] bf16 bits: the projection's data operand (split)
    const uint16_t* x_lo = nullptr;
    const float* wall3 = nullptr;     // [T][kc]
    int kc = 0;                       // K * C, a multiple of 8
};

// Scratch of the matching loop (device), per batch.
struct MatchScratch {
    float* cfmax;      // [nb][W]   per-sample maximum (windows longer than the staged chunk)
    int* at_t;         // [nb][W]   template of the spike accepted at w this iteration, -1 if none
    float* at_amp;     // [nb][W]
    MatchRescore rs;   // exact re-score of accepted candidates (rs.bt0 null: off)
};

// One spike record as written by the feature kernel (host-mapped memory).
struct SpikeRec {
    int32_t batch, w, t, iter;
    float amp, x, y;
    int32_t cluster;
    float feat[64];
};

constexpr int kMatchThreads = 512;       // matching loop, scores in L2 (two CTAs per SM)
constexpr int kMatchThreadsSmem = 768;   // matching loop, scores in shared memory (one CTA per SM)
constexpr int kMatchThreadsWide = 1024;  // matching loop, scores in L2, 16-CTA clusters, one CTA per SM

// output times per tile of the tensor-core high-pass (the band matrix is tile x Kt): 256 for
// groups of batches (the window tiles are re-read half as often), 128 for a few batches (twice
// the CTAs for one window)
constexpr int kHighpassTileSmall = 128, kHighpassTileLarge = 256, kHighpassSmallGroup = 8;

// raise (never lower) a kernel's dynamic shared-memory limit on the current device
cudaError_t raise_smem_limit(const void* kernel, size_t bytes);

// per-(window, channel) means (FP32) from exact integer sums; colsum [nb][C] and ticket
// [nb][ceil(C / 256)] must be zero before the first launch and are zero again after each launch
void launch_colsum(const int16_t* raw, int64_t row_stride, const int32_t* chan, int C, int W, int NT,
                   int nb, long long* colsum, int* ticket, float* mean, cudaStream_t s);
void launch_car(const int16_t* raw, int64_t row_stride, const int32_t* chan, int C, int W, int NT, int nb,
                const float* mean, int L, int R, float* Xw, cudaStream_t s);
// channel-major, tf32-split variant feeding the tensor-core high-pass: Xt[(b, c)][pitch]
// bf16: Xt_hi / Xt_lo receive the BF16 split (viewed as bf16 arrays)
void launch_car_t(const int16_t* raw, int64_t row_stride, const int32_t* chan, int C, int W, int NT, int nb,
                  const float* mean, int L, int R, int pitch, float* Xt_hi, float* Xt_lo, cudaStream_t s,
                  bool bf16 = false);
// Ylo != nullptr: Y receives tf32(y) and Ylo the remainder (operands of the tensor-core GEMM)
void launch_highpass(const float* Xw, int C, int W, int L, int R, const float* taps, int nb, float* Y,
                     cudaStream_t s, float* Ylo = nullptr);

// stateful high-pass mode (kernels_iir.cu): a causal Butterworth high-pass as second-order sections
// with FP32 state per channel, then the median CAR, written to Y in the whitening GEMM's format
constexpr int kIirMaxSections = 2;   // orders up to 4
constexpr int kHighpassOrder = 3;    // Kilosort's high-pass: butter(3, fc, 'high') (preprocessing.py:121-136)
constexpr int kIirChunk = 32;        // rows per chunk of the chunked recurrence
struct IirCoeffs {
    int ns;                          // sections (unused ones are identity)
    float b[kIirMaxSections][3];     // b0, b1, b2 of each section
    float a[kIirMaxSections][2];     // a1, a2 (a0 = 1)
    float zi[2 * kIirMaxSections];   // state of the steady response to a unit constant input
    float P[4 * kIirMaxSections * kIirMaxSections];   // zero-input state transition over kIirChunk rows
};
// the rows of one group: window b = rows [b NT, b NT + W); independent: every window is its own
// chain (windows API), else the group is one chain of span rows whose entering state is carried
// (reset: a segment starts, the steady state of the first row instead); carry_row: the row whose
// entering state the next group continues from (nb NT)
struct IirGroup {
    int nb, W, NT, span;
    bool independent, reset;
    int carry_row;
    int chunks;   // set by the launcher
};
// sections (b0, b1, b2, 1, a1, a2) of a Butterworth high-pass; returns their count, -1 on bad args
int butter_highpass_sos(int order, double fc, double fs, std::vector<double>& sos);
// the coefficients, and the powers P^0 .. P^kIirChunk of the chunk transition ([kIirChunk + 1][4][4])
IirCoeffs make_iir_coeffs(const std::vector<double>& sos, std::vector<float>& powers);
int iir_chunks(const IirGroup& g);
// pw: the powers of make_iir_coeffs on the device; zs, sin: [iir_chunks(g)][C] float4 scratch;
// carried [C] float4 (read on continuation, written at carry_row); out_mode 0 = FP32 Y, 1 = TF32
// split (Ylo may be null: tf32 alone), 2 = BF16 split
cudaError_t launch_iir_car(const int16_t* raw, int64_t row_stride, const int32_t* chan, int C, IirGroup g,
                           const IirCoeffs& k, const float* pw, float4* zs, float4* sin, float4* carried, float* Y,
                           float* Ylo, int out_mode, cudaStream_t s, int64_t& nl);

void launch_sgemm_nt(const float* A, int64_t lda, int64_t strideA, const float* B, int64_t ldb,
                     float* Cm, int64_t ldc, int64_t strideC, int M, int N, int K, int nb, cudaStream_t s);
// wPCA_host (K*nt floats) enables the specialisation with the basis in the parameter bank;
// Blo != nullptr writes the tf32 split like launch_highpass.
void launch_basis_conv_host(const float* Z, int C, int W, const float* wPCA_dev, const float* wPCA_host, int K,
                            int nt, int nb, float* Bpc, cudaStream_t s, float* Blo = nullptr,
                            bool round_tf32 = false);

// tensor-core (tcgen05) FP32-accurate GEMM C[m][n] = sum_k A[m][k] B[n][k] from tf32-split operands
struct UmmaOperands;
UmmaOperands* umma_make(const float* a_hi, const float* a_lo, int64_t rows_a, const float* b_hi, const float* b_lo,
                        int64_t rows_b, int K);
void umma_free(UmmaOperands* u);
cudaError_t launch_umma_gemm(const UmmaOperands* u, float* Cm, int M, int N, int64_t ldc, int* err, cudaStream_t s);
// the same with K split S ways across CTAs (for launches too small to fill the GPU): partial tiles in
// ws [S][M][ldc], then summed in slice order into C (deterministic)
cudaError_t launch_umma_gemm_splitk(const UmmaOperands* u, float* Cm, int M, int N, int64_t ldc, float* ws, int S,
                                    int* err, cudaStream_t s);
// circular high-pass on the tensor cores: x = channel-major windows [rows][cols] (tf32 split),
// g = the 128 x K band matrix of the taps (tf32 split)
UmmaOperands* umma_make_toeplitz(const float* x_hi, const float* x_lo, int64_t rows, int64_t cols, int tile, const float* g_hi,
                                 const float* g_lo, int K);
cudaError_t launch_umma_highpass(const UmmaOperands* u, float* Y_hi, float* Y_lo, int nb, int C, int W, int* err,
                                 cudaStream_t s);
// the same on BF16 splits (x: bf16 [rows][cols], cols % 8 == 0; g: bf16 [tile][K], K % 32 == 0); its
// epilogue writes Y as the BF16 split (Y_hi / Y_lo viewed as bf16)
UmmaOperands* umma_make_toeplitz_bf16(const void* x_hi, const void* x_lo, int64_t rows, int64_t cols, int tile,
                                      const void* g_hi, const void* g_lo, int K);
void launch_split_tf32(const float* x, float* hi, float* lo, int64_t n, cudaStream_t s);
// BF16 split: hi = bf16(x), lo = bf16(x - hi) (bf16 arrays of n elements)
void launch_split_bf16(const float* x, void* hi, void* lo, int64_t n, cudaStream_t s);
// FP8 projection operands (kernels_lowp.cu).  Calibration, once: from the rows of a BF16-split data
// operand x [rows][kc], the per-column scales sig / isig [kc] and the folded e4m3 templates w8
// [T][kc] with their scales tscale [T] (colmax [kc] scratch).  Quantize: x8 = e4m3(x * isig).
void launch_lowp_calibrate(const void* x_hi, const void* x_lo, int64_t rows, int kc, const float* wall3, int T,
                           unsigned* colmax, float* sig, float* isig, uint8_t* w8, float* tscale, cudaStream_t s);
void launch_lowp_quantize(const void* x_hi, const void* x_lo, int64_t rows, int kc, const float* isig, uint8_t* x8,
                          cudaStream_t s);
// one low-precision product: lowp 1 = A, B bf16 [rows][K] (kind::f16, K % 32 == 0), 2 = A, B FP8 e4m3
// bytes [rows][K] (kind::f8f6f4, K % 64 == 0); col_scale (may be null) scales column n of C by
// col_scale[n] in the epilogue
UmmaOperands* umma_make_lowp(const void* a, int64_t rows_a, const void* b, int64_t rows_b, int K, int lowp,
                             const float* col_scale);
// the GEMM on BF16-split operands (kind::f16, hi*hi + hi*lo + lo*hi; K % 32 == 0)
UmmaOperands* umma_make_bf16(const void* a_hi, const void* a_lo, int64_t rows_a, const void* b_hi, const void* b_lo,
                             int64_t rows_b, int K);
// the same GEMM, whose epilogue also writes the result channel-major, Zt[(row / wlen) * N + n][row %
// wlen] at row pitch zpitch, as its tf32 split (zt_lo may be null: tf32 alone), or as its BF16
// split into zt_hi / zt_lo viewed as bf16 arrays when zt_bf16
cudaError_t launch_umma_gemm_zt(const UmmaOperands* u, float* Cm, int M, int N, int64_t ldc, float* zt_hi,
                                float* zt_lo, int wlen, int zpitch, int* err, cudaStream_t s, bool zt_bf16 = false);

// temporal basis convolution on the tensor cores (kernels_umma.cu): Bpc[b][w][k][c] from the
// channel-major whitened windows Zt[(b, c)][time] and the components' band tiles of every K-step
struct ConvGeometry {
    bool bf16 = false;  // operands are BF16 splits (kind::f16) instead of TF32 splits
    int step = 16;      // input times per K-step: 64-byte rows, 16 fp32 or 32 bf16
    int tw = 32;        // output times per tile
    int ks = 0;         // K-steps per tile
    int hr = 0;         // a tile's first input time is its first output time - hr (16-byte aligned)
    int kg = 0;         // components per tile: one MMA of N = kg * tw columns per K-step and product
    int ncg = 0;        // component groups (tiles of one (rows, times) block)
    int rows = 0;       // band rows, ncg * ks * kg * tw (the band array is [rows][step])
};
bool conv_tc_geometry(int nt, int K, ConvGeometry& g, bool bf16 = false);
// band[cg][s][g tw + j][i] = wPCA[cg kg + g][step s + i - j - (hr - nt / 2)] (zero outside
// 0..nt-1 and for components >= K): the B operand of K-step s, [rows][step]
void conv_tc_bands(const float* wPCA, int K, int nt, const ConvGeometry& g, float* bands);
struct ConvOperands;
ConvOperands* conv_tc_make(const float* zt_hi, const float* zt_lo, int64_t rows, int wlen, int zpitch,
                           const float* s_hi, const float* s_lo, int K, const ConvGeometry& g);
void conv_tc_free(ConvOperands* u);
// out_lo == nullptr: store tf32(x) when hi_only, else fp32 x; out_bf16: the BF16 split of x into
// out_hi / out_lo viewed as bf16 arrays
cudaError_t launch_umma_basis_conv(const ConvOperands* u, float* out_hi, float* out_lo, bool hi_only, int nb, int C,
                                   int W, int* err, cudaStream_t s, bool out_bf16 = false);
cudaError_t launch_match(float* Bt, float* Xres, const float* ctcP, const float* pre_wf, const float* nm,
                         float th2, int W, int T, int C, int nt, int max_iters, int nb,
                         const MatchScratch& sc, const MatchOut& out, cudaStream_t s, int variant = 0,
                         bool residual = true);
// the residual after a matching loop: Xres[w][:] -= amp * waveform[t][w - w_s + nt/2][:] for the
// spikes of out, in list order
cudaError_t launch_residual(float* Xres, const float* pre_wf, const MatchOut& out, int W, int C, int nt, int nb,
                            cudaStream_t s);

// pruned matching tier (kernels_prune.cu): per sample the keep (<= kPruneKeepMax) templates of
// largest initial Cf, lists lrk / lsc [nb][W][kPruneKeepMax]; the loop on those lists
constexpr int kPruneKeepMax = 32;
constexpr uint16_t kListPad = 0xffffu;   // an unused list entry (a sample whose list is shorter)
constexpr int kPruneThreads = 1024;
void launch_prune_select(const float* Bt, const float* nm, int nb, int W, int T, int keep, uint16_t* lrk, float* lsc,
                         cudaStream_t s, int keep_wide = 0, float crowd_cf = 0.f);
// cf_scratch [nb][W + 2nt] and slot_scratch [nb][W] hold the per-sample maxima of windows whose
// maxima do not fit in shared memory (prune_mode without bit 0); may be null otherwise
cudaError_t launch_match_pruned(const uint16_t* lrk, float* lsc, int keep, const float* ctcP, const float* nm,
                                float th2, int W, int T, int nt, int max_iters, int nb, float* cf_scratch,
                                unsigned char* slot_scratch, const MatchOut& out, cudaStream_t s);
// where a window's per-sample state lives: bit 0 = maxima in shared memory, bit 1 = listed
// templates too, bit 2 = their scores too; 0 = maxima in the caller's scratch; -1 = too large for
// the tier
int prune_mode(int W, int T, int nt, int keep);

void launch_features(const float* Xres, const MatchOut& out, int nb, int W, int C, int T, int K, int nt, int nC,
                     const float* wPCA, const int64_t* iCC, const int64_t* iU, const float* Ucc, const float* xc,
                     const float* yc, const float* centroids, int n_final, const float* cpca, const float* cpca_nm,
                     float r2, const int* rec_offset, SpikeRec* recs, int batch_base, cudaStream_t s);
// the same records from the basis convolution Bpc [b][w][k][c] (fmt 0: fp32; 1: fp32 pair hi + lo;
// 2: BF16 pair) and the accepted spikes, without the residual; xcorr = basis_xcorr(wPCA) on the
// device, wall3t = Wall3 channel-major [T][C][K]
void basis_xcorr(const float* wPCA, int K, int nt, float* P);   // P [K][K][2 nt - 1]
void launch_features_direct(const void* bpc_hi, const void* bpc_lo, int fmt, const MatchOut& out, int nb, int W,
                            int C, int T, int K, int nt, int nC, const float* wall3t, const float* xcorr,
                            const int64_t* iCC, const int64_t* iU, const float* Ucc, const float* xc, const float* yc,
                            const float* centroids, int n_final, const float* cpca, const float* cpca_nm, float r2,
                            const int* rec_offset, SpikeRec* recs, int batch_base, cudaStream_t s);
void launch_rec_offsets(const MatchOut& out, int nb, int* rec_offset, cudaStream_t s);

}  // namespace lss
