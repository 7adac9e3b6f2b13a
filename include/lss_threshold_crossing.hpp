// lss_threshold_crossing.hpp -- C++ drop-in for the reference's threshold-crossing sorter.
//
// Mirrors src/SpikeSorter/ThresholdCrossing.h:17-93 (constructor from InputParameters + a
// DataSocket, runThresholdCrossing(), getChannelCount()) over the C ABI of lss_threshold.h.
// Differences from the reference, by design:
//   * the per-channel means and medians are constructor arguments (the reference compiles in
//     constants measured on one recording, ThresholdCrossing.cpp:157,182; lss_tc_calibrate
//     computes them from a block of rows the way its commented-out code did);
//   * fetches deliver int16 rows and the test runs on the GPU;
//   * events carry the stream sample of their own row (the reference adds the row index to the
//     stream count read before the fetch, ThresholdCrossing.cpp:207,224);
//   * no UDP handshake (ThresholdCrossing.cpp:53-79); events go to an EventSink callback and to
//     SpikeOutput_TC.txt lines "%20ld,%4ld,%f" = time, channel, 0 (ThresholdCrossing.cpp:194,227).
#pragma once

#include <cstdio>
#include <functional>
#include <vector>

#include "lss_online_spikes_v2.hpp"
#include "lss_threshold.h"

namespace lss {

using EventSink = std::function<void(const lss_tc_event* events, int64_t n)>;

class ThresholdCrossing {
public:
    // params: iNumTemplates = channels per row, fThresholdStd, iMinScanWindow / iMaxScanWindow
    // (fetch sizes), uSelectedDevice, sOSSOutputFolder ("" = no SpikeOutput_TC.txt)
    ThresholdCrossing(const InputParameters& params, const std::vector<float>& means,
                      const std::vector<float>& medians, DataSocket* socket, EventSink sink = nullptr);
    ~ThresholdCrossing();
    ThresholdCrossing(const ThresholdCrossing&) = delete;
    ThresholdCrossing& operator=(const ThresholdCrossing&) = delete;

    // The loop of ThresholdCrossing.cpp:195-252: wait for iMinScanWindow new rows, fetch what
    // arrived (the newest iMaxScanWindow when more), test it, emit the events.  Returns when the
    // socket stops running or stop() was called.
    void runThresholdCrossing();
    void stop() { running_ = false; }

    long getChannelCount() const { return c_; }
    lss_tc_handle* handle() const { return h_; }
    int64_t eventsWritten() const { return written_; }

private:
    void emit();
    lss_tc_handle* h_ = nullptr;
    InputParameters params_;
    DataSocket* sock_ = nullptr;
    EventSink sink_;
    OSSSpecificParams os_;
    std::FILE* out_ = nullptr;
    std::vector<int16_t> buf_;
    std::vector<lss_tc_event> ev_;
    volatile bool running_ = true;
    int64_t written_ = 0;
    int c_ = 0;
};

}  // namespace lss
