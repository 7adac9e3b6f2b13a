/*
 * lss_threshold.h -- C ABI of the GB300 threshold-crossing detector, the reference's second
 * sorter type (InputParameters.iSorterType == 1, src/main.cpp:87-89; class ThresholdCrossing,
 * src/SpikeSorter/ThresholdCrossing.h:17-93).
 *
 * Per fetched block of int16 rows [n_rows][n_chan] (channel fastest) the reference computes, on
 * the host, for every channel c and row j (ThresholdCrossing.cpp:209-226):
 *     y = (float)x[j][c] - means[c]                      (float32 subtraction)
 *     event if  (double)y <= -1.0 * (double)threshold_std * (double)medians[c]
 * and emits the events channel by channel, rows in order within a channel, each with template =
 * channel and amplitude 0 (ThresholdCrossing.cpp:223-228).  Here a handle runs that test on the
 * GPU: the float comparison is turned once, exactly, into an integer threshold per channel
 * (lss_tc_int_thresholds), each push is scanned by device kernels and its events come back in the
 * reference's order.  Events carry the true stream sample of their row; the reference stamps row
 * j with the stream count read before the fetch plus j (ThresholdCrossing.cpp:207,224), i.e. the
 * newest sample of the fetch, which shifts every event by the fetch length -- that offset is not
 * reproduced.  Status codes are those of lss_gb300.h.
 */
#ifndef LSS_THRESHOLD_H
#define LSS_THRESHOLD_H

#include <stdint.h>

#include "lss_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define LSS_TC_ABI_VERSION 1
#define LSS_TC_MAX_CHANNELS 4096

typedef struct lss_tc_params {
    int32_t abi_version;    /* = LSS_TC_ABI_VERSION */
    int32_t device;         /* CUDA ordinal */
    int32_t n_chan;         /* channels per row (ThresholdCrossing m_lC = InputParameters.iNumTemplates) */
    float threshold_std;    /* InputParameters.fThresholdStd (the GUI's default is 3, InputGui.cpp:102) */
    int64_t max_rows;       /* largest push (rows); the reference's fetch limit iMaxScanWindow; default 1500 */
    int64_t event_cap;      /* events kept per push; 0 = max(4096, max_rows * n_chan / 16) */
    int32_t profile;        /* 1 = time each stage with CUDA events (lss_tc_stage_times) */
    int32_t reserved[5];
} lss_tc_params;

/* One threshold crossing.  The reference sends (time, template = channel, amplitude = 0) in its
 * OnlineSpikesPayload (ThresholdCrossing.cpp:238-246); value is the mean-removed sample y. */
typedef struct lss_tc_event {
    int64_t time;       /* stream sample of the row */
    int32_t channel;    /* channel index within the row */
    float value;        /* y = (float)x - means[channel] */
} lss_tc_event;

typedef struct lss_tc_handle lss_tc_handle;

int lss_tc_default_params(lss_tc_params* p);

/* The integer form of the reference's test, computed on the host without a GPU: out[c] = the
 * largest int16 x with (double)((float)x - means[c]) <= -1.0 * (double)threshold_std *
 * (double)medians[c], or -32769 when no int16 value crosses.  Because the float subtraction is
 * monotone in x, "x <= out[c]" is the same test bit for bit. */
int lss_tc_int_thresholds(int32_t n_chan, const float* means, const float* medians, float threshold_std,
                          int32_t* out);

/* Per-channel statistics of a block of rows, as the reference's commented-out calibration
 * computes them (ThresholdCrossing.cpp:146-177): means[c] = (float)sum / (float)n_rows (the sum
 * exact in int64), medians[c] = element n_rows/2 of the sorted |(float)x - means[c]|.  Host
 * only; the reference ships constants measured this way (ThresholdCrossing.cpp:157,182). */
int lss_tc_calibrate(const int16_t* rows, int64_t n_rows, int32_t n_chan, float* means, float* medians);

/* Allocate a detector for n_chan channels with per-channel means and medians (copied).
 * Replaces ThresholdCrossing::ThresholdCrossing (ThresholdCrossing.cpp:21-99) minus its UDP
 * handshake. */
int lss_tc_open(const lss_tc_params* p, const float* means, const float* medians, lss_tc_handle** out);

/* Scan n_rows int16 rows [n_rows][n_chan]; row 0 is stream sample first_row_sample.  The rows
 * are copied into pinned staging before the call returns; the scan runs asynchronously on the
 * handle's stream.  n_rows <= max_rows.  Replaces the fetch + DC removal + test loops of
 * runThresholdCrossing (ThresholdCrossing.cpp:207-230). */
int lss_tc_push(lss_tc_handle* h, const int16_t* rows, int64_t n_rows, int64_t first_row_sample);

/* The same for rows already in device memory on the handle's device; they must stay valid until
 * the push is collected (lss_tc_poll / lss_tc_pending). */
int lss_tc_push_device(lss_tc_handle* h, const int16_t* dev_rows, int64_t n_rows, int64_t first_row_sample);

/* Copy out events push by push, each push in the reference's order (channel, then row).  Blocks
 * until the oldest push in flight is done when the queue is empty.  *n_out = events written; the
 * rest stay queued.  A push with more than event_cap events keeps the first event_cap and this
 * call returns LSS_ERR_OVERFLOW once, after delivering what fits. */
int lss_tc_poll(lss_tc_handle* h, lss_tc_event* out, int64_t cap, int64_t* n_out);

/* Events waiting after all pushes in flight are done. */
int lss_tc_pending(lss_tc_handle* h, int64_t* n);

/* The handle's integer thresholds (n = n_chan). */
int lss_tc_thresholds(const lss_tc_handle* h, int32_t* out, int32_t n);

/* The handle's CUDA stream (a cudaStream_t) as an opaque pointer. */
int lss_tc_cuda_stream(const lss_tc_handle* h, void** stream);

/* Device kernels launched by the last push. */
int lss_tc_kernel_launches(const lss_tc_handle* h, int64_t* n);

/* Device time per stage accumulated with CUDA events (profile = 1): ms[0..4] = h2d, count,
 * offsets, emit, d2h (the copy of the events to host memory); *n_pushes = pushes timed. */
#define LSS_TC_N_STAGES 5
int lss_tc_stage_times(lss_tc_handle* h, double* ms, int32_t n, int64_t* n_pushes);

/* Free the detector (ThresholdCrossing::~ThresholdCrossing, ThresholdCrossing.cpp:109-118). */
int lss_tc_close(lss_tc_handle* h);

/* Message of the last failure on h, or of the last failed handle-less call on this thread. */
const char* lss_tc_last_error(const lss_tc_handle* h);

#ifdef __cplusplus
}
#endif
#endif /* LSS_THRESHOLD_H */
