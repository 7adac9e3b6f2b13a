// payload.cpp -- the per-batch spike message in the reference's cereal binary layout
// (include/lss_payload.h).  Host code only: a message is a few kilobytes, built once per batch
// from the spikes lss_poll returns, off the GPU's path.
#include "../../include/lss_payload.h"

#include <cstring>
#include <limits>

namespace {

// little-endian raw bytes of a value (the layout is fixed whatever the host's byte order)
template <typename T>
uint8_t* put(uint8_t* p, T v) {
    unsigned char b[sizeof(T)];
    std::memcpy(b, &v, sizeof(T));
    const uint16_t probe = 1;
    const bool little = *reinterpret_cast<const unsigned char*>(&probe) == 1;
    for (size_t i = 0; i < sizeof(T); ++i) p[i] = little ? b[i] : b[sizeof(T) - 1 - i];
    return p + sizeof(T);
}

template <typename T>
const uint8_t* get(const uint8_t* p, T* v) {
    unsigned char b[sizeof(T)];
    const uint16_t probe = 1;
    const bool little = *reinterpret_cast<const unsigned char*>(&probe) == 1;
    for (size_t i = 0; i < sizeof(T); ++i) b[i] = little ? p[i] : p[sizeof(T) - 1 - i];
    std::memcpy(v, b, sizeof(T));
    return p + sizeof(T);
}

uint8_t* put_long(uint8_t* p, int64_t v, int lb) {
    if (lb == 8) return put<int64_t>(p, v);
    return put<uint32_t>(p, (uint32_t)(uint64_t)v);   // the low 32 bits, as a 32-bit long holds them
}

const uint8_t* get_long(const uint8_t* p, int64_t* v, int lb) {
    if (lb == 8) return get<int64_t>(p, v);
    int32_t x;
    p = get<int32_t>(p, &x);
    *v = x;
    return p;
}

// fixed bytes around the three vectors: 2 longs + 3 counts + double + float + 2 longs + 4 int16 + double
int64_t fixed_bytes(int lb) { return 2 * lb + 3 * 8 + 8 + 4 + 2 * lb + 4 * 2 + 8; }

}  // namespace

extern "C" {

int lss_payload_size(int64_t n_spikes, int32_t long_bytes, int64_t* bytes) {
    if (!bytes || n_spikes < 0 || (long_bytes != 4 && long_bytes != 8)) return LSS_ERR_ARG;
    if (n_spikes > (std::numeric_limits<int64_t>::max() - 64) / (2 * long_bytes + 4)) return LSS_ERR_ARG;
    *bytes = fixed_bytes(long_bytes) + n_spikes * (2 * long_bytes + 4);
    return LSS_OK;
}

int lss_payload_serialize(const lss_payload_header* hdr, const lss_spike* spikes, int64_t n_spikes,
                          int32_t long_bytes, uint8_t* out, int64_t cap, int64_t* n_out) {
    int64_t need = 0;
    if (!hdr || !n_out || (n_spikes > 0 && !spikes)) return LSS_ERR_ARG;
    const int st = lss_payload_size(n_spikes, long_bytes, &need);
    if (st != LSS_OK) return st;
    *n_out = need;
    if (!out || cap < need) return LSS_ERR_ARG;
    const int lb = long_bytes;
    uint8_t* p = out;
    p = put_long(p, hdr->recording_offset, lb);
    p = put_long(p, hdr->stream_sample_ct, lb);
    p = put<uint64_t>(p, (uint64_t)n_spikes);
    for (int64_t i = 0; i < n_spikes; ++i) p = put_long(p, spikes[i].time, lb);
    p = put<uint64_t>(p, (uint64_t)n_spikes);
    for (int64_t i = 0; i < n_spikes; ++i) p = put_long(p, spikes[i].cluster, lb);
    p = put<uint64_t>(p, (uint64_t)n_spikes);
    for (int64_t i = 0; i < n_spikes; ++i) p = put<float>(p, spikes[i].amp);
    p = put<double>(p, hdr->vrms);
    p = put<float>(p, hdr->p2p);
    p = put_long(p, hdr->process_time, lb);
    p = put_long(p, hdr->event_stream_sample_ct, lb);
    p = put<int16_t>(p, hdr->predict_label);
    p = put<int16_t>(p, hdr->label);
    p = put<int16_t>(p, hdr->n_trials);
    p = put<int16_t>(p, hdr->n_correct);
    p = put<double>(p, hdr->confidence);
    return p - out == need ? LSS_OK : LSS_ERR_INTERNAL;
}

int lss_payload_parse(const uint8_t* buf, int64_t len, int32_t long_bytes, lss_payload_header* hdr,
                      int64_t* times, int64_t* templates, float* amps, int64_t cap, int64_t* n_spikes) {
    if (!buf || !hdr || !n_spikes || len < 0 || cap < 0 || (long_bytes != 4 && long_bytes != 8)) return LSS_ERR_ARG;
    const int lb = long_bytes;
    if (len < fixed_bytes(lb)) return LSS_ERR_ARG;
    const uint8_t* p = buf;
    const uint8_t* end = buf + len;
    lss_payload_header h{};
    p = get_long(p, &h.recording_offset, lb);
    p = get_long(p, &h.stream_sample_ct, lb);
    uint64_t counts[3];
    const int widths[3] = {lb, lb, 4};
    const uint8_t* data[3];
    for (int v = 0; v < 3; ++v) {
        if (end - p < 8) return LSS_ERR_ARG;
        p = get<uint64_t>(p, &counts[v]);
        if (counts[v] > (uint64_t)(end - p) / (uint64_t)widths[v]) return LSS_ERR_ARG;
        data[v] = p;
        p += counts[v] * widths[v];
    }
    if (counts[0] != counts[1] || counts[1] != counts[2]) return LSS_ERR_ARG;
    if (end - p != 8 + 4 + 2 * lb + 4 * 2 + 8) return LSS_ERR_ARG;
    p = get<double>(p, &h.vrms);
    p = get<float>(p, &h.p2p);
    p = get_long(p, &h.process_time, lb);
    p = get_long(p, &h.event_stream_sample_ct, lb);
    p = get<int16_t>(p, &h.predict_label);
    p = get<int16_t>(p, &h.label);
    p = get<int16_t>(p, &h.n_trials);
    p = get<int16_t>(p, &h.n_correct);
    p = get<double>(p, &h.confidence);
    const int64_t n = (int64_t)counts[0];
    const int64_t m = n < cap ? n : cap;
    for (int64_t i = 0; i < m; ++i) {
        if (times) get_long(data[0] + i * lb, &times[i], lb);
        if (templates) get_long(data[1] + i * lb, &templates[i], lb);
        if (amps) get<float>(data[2] + i * 4, &amps[i]);
    }
    *hdr = h;
    *n_spikes = n;
    return LSS_OK;
}

int lss_batch_p2p(const int16_t* rows, int64_t n_rows, int32_t n_chan, float* p2p) {
    if (!rows || !p2p || n_rows <= 0 || n_chan <= 0) return LSS_ERR_ARG;
    int lo = rows[0], hi = rows[0];
    const int64_t n = n_rows * (int64_t)n_chan;
    for (int64_t i = 1; i < n; ++i) {
        const int v = rows[i];
        lo = v < lo ? v : lo;
        hi = v > hi ? v : hi;
    }
    *p2p = (float)hi - (float)lo;
    return LSS_OK;
}

}  // extern "C"
