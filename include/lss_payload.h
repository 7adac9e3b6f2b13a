/*
 * lss_payload.h -- the per-batch spike message in the reference's wire format (host only).
 *
 * The reference sends one OnlineSpikesPayload per sorted batch to its decoder
 * (src/SpikeSorter/OnlineSpikesV2.cu:827-838), serialized by serialize<T>()
 * (src/Networking/SerializationHelpers.h:10-18) with cereal's BinaryOutputArchive, field by field
 * in the order of OnlineSpikesPayload::serialize (src/Networking/onlineSpikesPayload.h:30-46):
 *
 *     recordingOffset        long
 *     streamSampleCt         long
 *     Times                  uint64 count, then count x long
 *     Templates              uint64 count, then count x long
 *     Amplitudes             uint64 count, then count x float
 *     VRMS                   double
 *     P2P                    float
 *     processTime            long
 *     eventStreamSampleCt    long
 *     predictLabel, label, nTrials, nCorrect     int16 each
 *     confidence             double
 *
 * Every value is written as its raw little-endian bytes with no padding; a vector is its element
 * count as a uint64 followed by the elements.  `long` is 4 bytes in the reference's Windows build
 * (LLP64) and 8 bytes on LP64 systems: long_bytes selects the width, and a value written as a
 * 4-byte long keeps its low 32 bits (two's complement), as a 32-bit long holds it.
 *
 * The sorter fills Times with the spikes' stream times, Templates with their final clusters
 * (closestCluster's ids, OnlineSpikesV2.cu:1189-1204) and Amplitudes with their amplitudes; the
 * reference leaves VRMS at 0 and the decoder-side fields (eventStreamSampleCt .. confidence) zero.
 * Status codes are those of lss_gb300.h.
 */
#ifndef LSS_PAYLOAD_H
#define LSS_PAYLOAD_H

#include <stdint.h>

#include "lss_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lss_payload_header {
    int64_t recording_offset;         /* recordingOffset */
    int64_t stream_sample_ct;         /* streamSampleCt: the newest stream sample of the batch */
    double vrms;                      /* VRMS */
    float p2p;                        /* P2P: max - min of the batch's raw samples (lss_batch_p2p) */
    int32_t reserved;
    int64_t process_time;             /* processTime */
    int64_t event_stream_sample_ct;   /* eventStreamSampleCt */
    int16_t predict_label, label, n_trials, n_correct;
    double confidence;
} lss_payload_header;

/* Bytes of the message for n_spikes spikes. */
int lss_payload_size(int64_t n_spikes, int32_t long_bytes, int64_t* bytes);

/* Serialize one message: Times = spikes[i].time, Templates = spikes[i].cluster, Amplitudes =
 * spikes[i].amp.  *n_out = the message's size; LSS_ERR_ARG (nothing written) when cap is smaller. */
int lss_payload_serialize(const lss_payload_header* hdr, const lss_spike* spikes, int64_t n_spikes,
                          int32_t long_bytes, uint8_t* out, int64_t cap, int64_t* n_out);

/* Parse one message of exactly len bytes (the decoder's side).  *n_spikes = the element count of
 * the three vectors (which must agree); min(count, cap) entries are written to each non-NULL
 * array.  LSS_ERR_ARG for a message that is truncated, has trailing bytes or unequal counts. */
int lss_payload_parse(const uint8_t* buf, int64_t len, int32_t long_bytes, lss_payload_header* hdr,
                      int64_t* times, int64_t* templates, float* amps, int64_t cap, int64_t* n_spikes);

/* P2P of a batch as the reference computes it on the fetched samples (P2P_calc,
 * OnlineSpikesV2.cu:1137-1146): the largest minus the smallest value of rows [n_rows][n_chan]. */
int lss_batch_p2p(const int16_t* rows, int64_t n_rows, int32_t n_chan, float* p2p);

#ifdef __cplusplus
}
#endif

#endif
