// payload_ref.cpp -- TEST INFRASTRUCTURE ONLY: serializes one spike message with the reference's
// own vendored cereal (External/cereal, BinaryOutputArchive), so that the restatement in
// payload_oracle.py and the library's lss_payload_serialize can be checked byte for byte.
//
// The message's fields and their order follow OnlineSpikesPayload::serialize
// (src/Networking/onlineSpikesPayload.h:30-46); that header itself includes the reference's
// Windows socket layer (SerializationHelpers.h -> Sock.h) and does not compile here.  `L` stands
// for the reference's `long`: int32_t as in its Windows (LLP64) build, int64_t on LP64.
//
// stdin (little-endian): int32 long_bytes; int64 recording_offset, stream_sample_ct; uint64 n;
// n x int64 times; n x int64 templates; n x float amps; double vrms; float p2p; int64 process_time;
// int64 event_stream_sample_ct; 4 x int16 (predict_label, label, n_trials, n_correct); double
// confidence.  stdout: the archive's bytes.
#include <cereal/archives/binary.hpp>
#include <cereal/types/vector.hpp>

#include <cstdint>
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

namespace {

template <typename L>
struct SpikeMessage {
    L recording_offset = 0, stream_sample_ct = 0;
    std::vector<L> times, templates;
    std::vector<float> amps;
    double vrms = 0;
    float p2p = 0;
    L process_time = 0, event_stream_sample_ct = 0;
    int16_t predict_label = 0, label = 0, n_trials = 0, n_correct = 0;
    double confidence = 0;

    template <class Archive>
    void serialize(Archive& ar) {
        ar(recording_offset, stream_sample_ct, times, templates, amps, vrms, p2p, process_time,
           event_stream_sample_ct, predict_label, label, n_trials, n_correct, confidence);
    }
};

template <typename T>
T rd() {
    T v{};
    if (std::fread(&v, sizeof(T), 1, stdin) != 1) throw std::runtime_error("short input");
    return v;
}

template <typename L>
std::string run() {
    SpikeMessage<L> m;
    m.recording_offset = (L)rd<int64_t>();
    m.stream_sample_ct = (L)rd<int64_t>();
    const uint64_t n = rd<uint64_t>();
    for (uint64_t i = 0; i < n; ++i) m.times.push_back((L)rd<int64_t>());
    for (uint64_t i = 0; i < n; ++i) m.templates.push_back((L)rd<int64_t>());
    for (uint64_t i = 0; i < n; ++i) m.amps.push_back(rd<float>());
    m.vrms = rd<double>();
    m.p2p = rd<float>();
    m.process_time = (L)rd<int64_t>();
    m.event_stream_sample_ct = (L)rd<int64_t>();
    m.predict_label = rd<int16_t>();
    m.label = rd<int16_t>();
    m.n_trials = rd<int16_t>();
    m.n_correct = rd<int16_t>();
    m.confidence = rd<double>();
    std::ostringstream ss;
    {
        cereal::BinaryOutputArchive ar(ss);
        ar(m);
    }
    return ss.str();
}

}  // namespace

int main() {
    try {
        const int32_t lb = rd<int32_t>();
        const std::string out = lb == 4 ? run<int32_t>() : run<int64_t>();
        std::fwrite(out.data(), 1, out.size(), stdout);
        return 0;
    } catch (const std::exception& e) {
        std::cerr << e.what() << "\n";
        return 1;
    }
}
