/*
 * lss_gb300.h -- C ABI of the GB300-native LiveSpikeSorter per-batch sorting path.
 *
 * One handle = one probe stream (one sorter instance of the reference) on one CUDA device,
 * with its own non-blocking CUDA stream and device-resident state.  Handles are independent
 * and may be driven from different host threads; a single handle is single-producer.
 *
 * Every function returns an int status (LSS_OK = 0); no C++ exception crosses this
 * boundary and nothing calls exit().  lss_last_error() gives the message of the last
 * failure on a handle.  No CUDA or torch type appears in a signature.
 *
 * Semantics of one batch follow Kilosort 4.0.13 as vendored in the reference
 * (src/Python/run_online_spikes/Lib/site-packages/kilosort/): io.py:757-790 (filter),
 * template_matching.py:128-202 (run_matching), template_matching.py:50-51,68 (features and
 * spike time), postprocessing.py:9-46 (duplicates, positions).
 */
#ifndef LSS_GB300_H
#define LSS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LSS_ABI_VERSION 3
#define LSS_MAX_PCFEAT 64 /* nearest channels x PCs carried per spike */

enum lss_status {
    LSS_OK = 0,
    LSS_ERR_ARG = 1,      /* bad argument / size */
    LSS_ERR_IO = 2,       /* file missing or unreadable */
    LSS_ERR_FORMAT = 3,   /* .npy word size / rank / shape mismatch, bad misc.txt */
    LSS_ERR_CUDA = 4,     /* CUDA runtime failure (message has the CUDA error string) */
    LSS_ERR_NOMEM = 5,    /* device or pinned allocation failed / over the memory budget */
    LSS_ERR_OVERFLOW = 6, /* a per-batch spike buffer overflowed (spikes beyond it dropped) */
    LSS_ERR_STATE = 7,    /* call not valid in the handle's state */
    LSS_ERR_INTERNAL = 8
};

/* Per-handle options.  Fill with lss_default_params() and override fields. */
typedef struct lss_params {
    int32_t abi_version;    /* = LSS_ABI_VERSION */
    int32_t device;         /* CUDA ordinal (InputParameters.uSelectedDevice) */
    int32_t batch_samples;  /* NT: new samples per batch (InputParameters.iMaxScanWindow), default 1500 */
    int32_t max_iters;      /* matching-pursuit iterations per batch, default 50 (OnlineSpikesV2.cu:933) */
    int32_t group_batches;  /* batches launched together, default 1 (lowest latency); larger = throughput */
    int32_t n_chan_in;      /* channels per input row; 0 = C of the oss_input; > C selects channelMap */
    int32_t hp_half_taps;   /* high-pass FIR half length; 0 = automatic: the shortest one beyond which every tap
                               of the window's filter is < 1e-8 of its centre tap (442 for Kilosort's 300 Hz filter at 30 kHz) */
    int32_t dedup;          /* 1 = drop same-cluster spikes within duplicate_spike_bins (default 1) */
    float th_override;      /* > 0 replaces Th_learned of misc.txt */
    int32_t spike_cap;      /* per-batch spike buffer; 0 = automatic (2 * max_iters * ceil(W / (nt + 1))) */
    int64_t mem_budget;     /* device bytes this handle may hold; 0 = no limit (admission check) */
    int32_t profile;        /* 1 = time every stage with CUDA events (lss_stage_times) */
    int32_t match_variant;  /* 0 = automatic; 1 = scores in L2, 8-CTA clusters; 2 = scores in shared memory;
                               3 = scores in L2, 16-CTA clusters of 1024 threads (one CTA per SM) */
    int32_t gemm_path;      /* 0 = tensor cores (tcgen05, 3xTF32 = FP32 accuracy) where shapes allow; 1 = FP32 SIMT;
                               2 = tensor cores with the data operands stored once as TF32 (two products; the
                               fixed matrices keep FP32 accuracy): faster, spike agreement with 0 measured;
                               3 = the high-pass, whitening, convolution and projection on BF16 splits
                               (hi = bf16(x), lo = bf16(x - hi), hi*hi + hi*lo + lo*hi in FP32: ~1e-5 relative
                               per product) at the BF16 rate, where C and K*C are multiples of 32 (the
                               high-pass and whitening need C, the convolution and projection K*C); a stage
                               whose shape does not allow it runs as on 0;
                               4 = as 3, but the projection is one BF16 product (hi*hi) and 5 = one FP8 e4m3
                               product (per-(component, channel) activation scales set from the first group
                               and folded into the templates, per-template scales in the epilogue), FP32
                               accumulation; every accepted candidate's amplitude is then recomputed from the
                               exact FP32 projection of the split operands (its running score corrected by
                               exact - low-precision initial score); spikes can differ where the
                               low-precision score ranks candidates differently (agreement measured); both
                               need the tensor-core convolution, K*C a multiple of 64 (5) and match_keep 0 */
    int32_t cluster_rule;   /* final cluster of a spike: 0 = nearest centroid in (x, y) (OnlineSpikesV2.cu:1058-1074);
                               1 = best PC score 2 tF.mu - |mu|^2 among the clusters within cluster_radius_um of the
                               spike (OnlineKilosort.py:233-284; cluster_centroids_pca.npy [T_final, nC*K]), -1 if none */
    float cluster_radius_um;  /* radius of rule 1; 0 = 80 um (OnlineKilosort.py:449) */
    int32_t match_keep;     /* 0 = Kilosort's matching loop over every template (default); 1..32 = the pruned tier:
                               per sample only the match_keep templates of largest initial Cf = relu(B)^2 / nm
                               are scored through the loop (same updates on them, so the spikes equal the full
                               loop's unless an unlisted template would have won; agreement measured) */
    int32_t highpass_mode;  /* 0 = Kilosort's zero-phase high-pass, circular over each batch window (preprocessing.py:
                               120-154, OnlineSpikesV2.cu:1006-1056; hp_filter.npy), after the mean removal and median
                               CAR (default); 1 = the same 3rd-order Butterworth (butter(3, highpass_hz, 'high')) run
                               forward as second-order sections over the stream with FP32 state per channel carried
                               from batch to batch on the device (starting at a segment's first sample in its steady
                               state), then the median CAR; no mean removal (the filter removes DC).  The windows API
                               filters each window alone. */
    float highpass_hz;      /* edge of mode 1 (default 300, Kilosort's) */
    float sample_rate_hz;   /* sample rate of mode 1 (default 30000) */
    int32_t match_keep_wide;  /* 0 = every sample lists match_keep templates; match_keep < n <= 32 = a crowded
                                 sample lists n: one whose match_keep-th largest initial Cf exceeds
                                 match_keep_crowd * Th^2 (the templates a larger overlapping spike outranks
                                 there are the ones a short list misses) */
    float match_keep_crowd;   /* the crowding threshold of match_keep_wide, in units of Th^2 (default 0.5) */
} lss_params;

/* One sorted spike.  time is the stream sample (Kilosort template_matching.py:68). */
typedef struct lss_spike {
    int64_t time;       /* stream sample of the spike */
    int32_t tmpl;       /* pre-clustered template id (row of Wall3), Kilosort iY */
    int32_t cluster;    /* final cluster: nearest centroid in (x, y) */
    float amp;          /* B[iY, iX] / nm[iY] */
    float x, y;         /* feature-energy weighted position (um) */
    int32_t batch;      /* batch index within the stream */
    int32_t n_feat;     /* = nearest_chans * n_pcs */
    int32_t iter;       /* matching iteration that accepted the spike */
    float pcfeat[LSS_MAX_PCFEAT]; /* [nearest_chans][n_pcs] PC features */
} lss_spike;

typedef struct lss_info {
    int32_t C;          /* channels */
    int32_t T;          /* pre-clustered templates (Wall3 rows) */
    int32_t T_final;    /* final clusters (templates.npy rows / centroids) */
    int32_t K;          /* PCs */
    int32_t nt;         /* template length */
    int32_t nC;         /* nearest channels */
    int32_t nt0min;
    int32_t dup_bins;
    float th;           /* Th_learned in use */
    int32_t NT;         /* new samples per batch */
    int32_t W;          /* window = NT + 2 nt */
    int32_t group_batches;
    int64_t device_bytes;   /* device memory held by the handle */
    int64_t batches_done;
    int64_t spikes_done;
} lss_info;

typedef struct lss_handle lss_handle;

/* Defaults. */
int lss_default_params(lss_params* p);

/* Load an oss_input/ directory (cnpy semantics: row-major, fortran_order ignored) and
 * allocate all device state.  Replaces OnlineSpikesV2::OnlineSpikesV2 + initializeSorter +
 * allocateMemory + initializeStaticMemory (src/SpikeSorter/OnlineSpikesV2.cu:248-281,
 * 322-382, 410-660) minus the UDP handshake (establishDecoderConnection, :384-406). */
int lss_open(const char* oss_dir, const lss_params* p, lss_handle** out);

/* Shapes and counters. */
int lss_get_info(const lss_handle* h, lss_info* info);

/* Load and check an oss_input/ directory on the host alone, without a GPU: every file, shape,
 * word size and cross-dimension that lss_open checks (the exporter's own checks,
 * run_online_spikes.py:598-672 and subset_templates.py:48-66, and the loaders' in
 * SorterHelpers.cpp:24-115).  Returns lss_open's status for the same directory under the
 * default lss_params (cluster_centroids_pca.npy, read only for cluster_rule = 1, is not checked);
 * info (may be NULL) receives C, T, T_final, K, nt, nC, nt0min, dup_bins and th, the other fields
 * 0.  The message is lss_last_error(NULL). */
int lss_validate_oss_input(const char* oss_dir, lss_info* info);

/* Template subsetting of an oss_input/ directory: keep only some preclustered templates so a
 * stream's device state and per-batch work shrink (admission of more streams under mem_budget).
 * Replaces the reference's subset_templates.py (src/Python/subset_templates.py:1-343) with this
 * library's own selection on the loader's shape model.  A template's footprint is its energy per
 * channel, sum_k Wall3[t][k][c]^2.  Candidates: every template, or (chan_lo <= chan_hi) those whose
 * strongest channel's probe channel (channelMap.npy) lies in [chan_lo, chan_hi] (chan_rule 0), or
 * that have any in-range channel with RMS >= overlap_frac of the strongest's (chan_rule 1).  Then at
 * most max_templates (0 = all candidates): by spikes per template in
 * spike_detection_templates.npy, ties by energy then index (rank 0; energy when the file is
 * absent), or by energy (rank 1).  The kept indices come back ascending. */
typedef struct lss_subset_spec {
    int32_t max_templates;
    int32_t rank;          /* 0 = activity, 1 = energy */
    int32_t chan_lo, chan_hi;
    int32_t chan_rule;     /* 0 = strongest channel in range, 1 = any channel above overlap_frac */
    float overlap_frac;    /* default 0.1 */
} lss_subset_spec;
void lss_subset_default_spec(lss_subset_spec* spec);   /* no cap, no channel range, rank 0, 0.1 */
/* The kept indices (keep may be NULL to ask for the count; LSS_ERR_OVERFLOW if cap is too small). */
int lss_subset_plan(const char* oss_dir, const lss_subset_spec* spec, int32_t* keep, int32_t cap,
                    int32_t* n_keep);
/* Write the subset directory out_dir (must not exist): Wall3, ctc (both template axes), iU, Ucc,
 * the preclustered waveforms cut, every other file copied, subset_manifest.json with the kept
 * indices.  A spike's tmpl from the subset directory indexes that list.  LSS_ERR_ARG when nothing
 * would be cut.  Messages via lss_last_error(NULL). */
int lss_subset_write(const char* in_dir, const char* out_dir, const lss_subset_spec* spec);

/* Push n_samples rows of int16 [n_samples][n_chan_in] (channel fastest, SpikeGLX order).
 * stream_sample_ct = stream index of row 0, or -1 for "continues the previous push"; a
 * discontinuity flushes the current segment and starts a new one (the skip / behind policy
 * of OnlineSpikesV2::runSpikeSorting, OnlineSpikesV2.cu:698-761).  The caller may reuse the
 * rows when the call returns: rows in page-locked memory (cudaHostAlloc / cudaHostRegister) are
 * copied straight to the device and the call waits for that copy; pageable rows are copied into
 * the handle's pinned staging.  Every batch whose window is complete is launched asynchronously
 * on the handle's stream.  Replaces DataSocket::fetchLatest / fetchFromPlace +
 * the H2D copy + the per-batch body of runSpikeSorting (dataSocket.cpp:103-171,
 * OnlineSpikesV2.cu:747-822). */
int lss_push_batch(lss_handle* h, const int16_t* samples, int64_t n_samples, int64_t stream_sample_ct);

/* Process the samples still buffered as a final batch (last sample replicated to fill the
 * window, Kilosort io.py:626-629). */
int lss_flush(lss_handle* h);

/* Copy out finished spikes in time order (blocking until the oldest launched batch group is
 * done, if any).  *n_out = number written; if cap is too small the rest stay queued and
 * *n_out = cap.  Replaces saveSpikes + writeSpikesToFile + the payload vectors
 * (OnlineSpikesV2.cu:1148-1205, onlineSpikesPayload.h:8-48). */
int lss_poll(lss_handle* h, lss_spike* out, int64_t cap, int64_t* n_out);

/* Number of finished spikes waiting in the queue after waiting for all launched work. */
int lss_pending(lss_handle* h, int64_t* n);

/* Free everything (OnlineSpikesV2::~OnlineSpikesV2, OnlineSpikesV2.cu:283-320). */
int lss_close(lss_handle* h);

/* Message of the last failure on h (or, when h is NULL, of the last failed call on this thread
 * that takes no handle: lss_open, lss_match_noalloc). */
const char* lss_last_error(const lss_handle* h);

/* Sort explicit windows without stream framing: windows = int16 [n_windows][W][n_chan_in].
 * Spikes of window i carry batch = i and time = the window sample shifted like Kilosort
 * (s - nt//2 + nt0min).  counts[i] = spikes of window i; out receives them window by window,
 * each window in (time, template) order, no duplicate removal.  Replaces
 * OnlineSpikesV2::kilosortMatchingPursuit + computeClosestClusters for one batch
 * (OnlineSpikesV2.cu:853-1001) with the preprocessing before it (:771-808). */
int lss_sort_windows(lss_handle* h, const int16_t* windows, int32_t n_windows, int32_t W,
                     lss_spike* out, int64_t cap, int64_t* counts);

/* Stage outputs of one window for parity checks (float32):
 *   LSS_STAGE_PREPROCESSED  [W][C]  after mean, median CAR, high-pass, (M @ Wrot)
 *   LSS_STAGE_SCORES        [W][T]  B before the matching loop (transposed)
 *   LSS_STAGE_RESIDUAL      [W][C]  Xres after the loop */
enum lss_stage { LSS_STAGE_PREPROCESSED = 1, LSS_STAGE_SCORES = 2, LSS_STAGE_RESIDUAL = 3 };
int lss_debug_stage(lss_handle* h, const int16_t* window, int32_t W, int32_t stage, float* out, int64_t out_len);

/* Device kernels launched by the last lss_push_batch / lss_push_device_span / lss_sort_windows /
 * lss_flush call. */
int lss_kernel_launches(const lss_handle* h, int64_t* n);

/* Sort n_batches batches whose samples are already in device memory: dev_rows = int16
 * [n_batches*NT + 2*nt][n_chan_in] on the handle's device; batch b uses rows
 * [b*NT, b*NT + NT + 2*nt) and its spikes get stream times from first_row_sample = the stream
 * sample of row 0 (so batch b covers new samples first_row_sample + nt + b*NT ...).  The rows must
 * stay valid until the batches are collected (lss_poll / lss_pending).  For acquisition that
 * lands on the GPU directly; no host staging copy.  Replaces the H2D copy of
 * OnlineSpikesV2::runSpikeSorting (OnlineSpikesV2.cu:747-761) for device-resident input. */
int lss_push_device_span(lss_handle* h, const int16_t* dev_rows, int64_t n_batches, int64_t first_row_sample);

/* The handle's CUDA stream (a cudaStream_t) as an opaque pointer, for callers that order their
 * own device work or timing events against the sorter's. */
int lss_cuda_stream(const lss_handle* h, void** stream);

/* Per-stage device time accumulated with CUDA events since the handle opened (profile = 1):
 * ms[0..LSS_N_STAGES-1] = h2d, colsum, car, highpass, whiten, basis_conv, project, match,
 * features, d2h; *n_groups = batch groups timed.  The reference's per-stage Timer
 * (Timer.h:7-21) prints nothing; this is its working counterpart. */
#define LSS_N_STAGES 10
int lss_stage_times(lss_handle* h, double* ms, int32_t n, int64_t* n_groups);

/* The second-order sections (b0, b1, b2, 1, a1, a2 each, sos[6 * n_sections]) of the Butterworth
 * high-pass that highpass_mode 1 runs: order 1..4, edge cutoff_hz < fs_hz / 2.  Kilosort designs the
 * same filter with scipy.signal.butter (preprocessing.py:121-136); this is the library's own design
 * (bilinear transform of the analog prototype), exported so a caller can check it.  Sections are
 * ordered by pole radius, the gain on the first. */
int lss_butter_highpass_sos(int32_t order, double cutoff_hz, double fs_hz, double* sos, int32_t cap_sections,
                            int32_t* n_sections);

/* The matching loop of one window on buffers the caller owns, allocating no memory.
 *
 * No counterpart in the reference.  For callers that cannot allocate device memory when they
 * sort -- a real-time acquisition thread that must not wait on the allocator, code confined to a
 * memory pool owned by another framework, or an application that already keeps the scores and
 * the residual in its own device buffers.  All pointers are device pointers on the current CUDA
 * device; stream is a cudaStream_t (NULL = legacy default stream); the call is asynchronous.
 *   scores          [W][T]  template scores (B transposed); consumed (overwritten)
 *   residual        [W][C]  preprocessed window in, Xres out
 *   ctc_perm        [T][2*nt+1][T]  ctc_perm[s][l][t] = ctc[t][s][l]
 *   waveforms       [T][nt][C]      preclustered_template_waveforms
 *   template_norms  [T]             sum of squares of each Wall3 template
 *   n_spikes        [1]     spikes accepted (may exceed cap; the lists then hold the first cap);
 *                           negative when the kernel reported a fault (-2: it did not run with the
 *                           thread-block cluster shape it was launched for) -- the lists are then
 *                           not valid
 *   spike_sample / spike_template / spike_amp / spike_iter  [cap]  in (iteration, sample) order
 * Its working memory is a fixed device array of LSS_NOALLOC_SCRATCH_BYTES inside the library
 * (held on every GPU that loads it until the process exits), enough for windows of at most
 * LSS_NOALLOC_MAX_SAMPLES samples; a larger W returns LSS_ERR_ARG.  A call outside stream capture
 * looks up that array's device address on the current device (again after a cudaDeviceReset); a
 * call on a capturing stream reuses the address found before, so the first call on a device must
 * come before any capture (else LSS_ERR_ARG).  All calls share the array: calls whose work
 * overlaps on the GPU race, so serialise them (one stream, or events).
 * Errors: LSS_ERR_ARG / LSS_ERR_CUDA, message via lss_last_error(NULL). */
#define LSS_NOALLOC_MAX_SAMPLES 16384
#define LSS_NOALLOC_SCRATCH_BYTES 196864
int lss_match_noalloc(float* scores, float* residual, const float* ctc_perm, const float* waveforms,
                      const float* template_norms, float th, int32_t W, int32_t T, int32_t C, int32_t nt,
                      int32_t max_iters, int32_t* n_spikes, int32_t* spike_sample, int32_t* spike_template,
                      float* spike_amp, int32_t* spike_iter, int32_t cap, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LSS_GB300_H */
