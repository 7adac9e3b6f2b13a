// lss_online_spikes_v2.hpp -- C++ drop-in for the reference's sorter class and its input socket.
//
// Mirrors src/SpikeSorter/OnlineSpikesV2.h:29-34 (constructor from InputParameters + a
// DataSocket, runSpikeSorting()) and src/SpikeSorter/dataSocket.h:17-57 (OSSSpecificParams,
// getStreamSampleCt / fetchLatest / fetchFromPlace / waitUntil), over the C ABI of lss_gb300.h.
// Differences from the reference, by design:
//   * fetch* deliver int16 rows (channel fastest) -- the GPU converts; the reference converts
//     to float on the host (dataSocket.cpp:122-124);
//   * no UDP handshake in the constructor (OnlineSpikesV2.cu:384-406); spikes go to a
//     SpikeSink callback and to spikeOutput.txt in the reference's line format
//     "time,cluster,amplitude,y" (OnlineSpikesV2.cu:1161-1164);
//   * errors throw lss::SorterError (status + message) instead of exit().
#pragma once

#include <climits>
#include <cstdint>
#include <fstream>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "lss_gb300.h"

namespace lss {

typedef unsigned long long t_ull;
enum streamTypes { NIDQ, OBX, IMEC };

// Parameters of one sorter's slice of the acquisition (dataSocket.h:17-21).
struct OSSSpecificParams {
    long lNChans = 0;
    std::vector<int> vImecChannels;
    int substream = 0;
};

// Acquisition interface (dataSocket.h:23-57), int16 flavour.  fetch* return the stream sample
// count one past the last row written and write at most maxRows rows to data.
class DataSocket {
public:
    virtual ~DataSocket() = default;
    virtual t_ull getStreamSampleCt(int streamType, const OSSSpecificParams& p) = 0;
    // rows [lStartCt, latest) clipped to maxRows (the newest maxRows when more are available)
    virtual t_ull fetchLatest(int16_t* data, long maxRows, const OSSSpecificParams& p, t_ull lStartCt) = 0;
    // rows [lStartCt, lStartCt + maxRows) clipped to what is available
    virtual t_ull fetchFromPlace(int16_t* data, long maxRows, const OSSSpecificParams& p, t_ull lStartCt) = 0;
    virtual void waitUntil(t_ull lCt, const OSSSpecificParams& p) { (void)lCt; (void)p; }
    // false once the source has nothing more to deliver (a file replay reached its end)
    virtual bool isRunning() { return true; }
};

// The fields of InputParameters (src/Networking/inputParameters.h:10-77) the sorter uses.
struct InputParameters {
    std::string sInputFolder;        // oss_input/ directory
    std::string sOSSOutputFolder;    // where spikeOutput.txt goes ("" = no file)
    uint16_t uSelectedDevice = 0;
    int iMinScanWindow = 82;
    int iMaxScanWindow = 1500;       // new samples per batch
    int iTimeBehind = 0;             // ms allowed behind; 0 = skip to the newest data when behind
    bool bSmallskip = false;
    float fImecSamplingRate = 30000.f;
    int iSubstream = 0;
    int iMaxIts = 50;
    int iGroupBatches = 1;
    int iChannelsIn = 0;             // row width delivered by the socket (0 = oss_input channels)
    // ThresholdCrossing (iSorterType 1): channels per row (ThresholdCrossing.cpp:26 reads them
    // from iNumTemplates) and the threshold in units of the per-channel median (fThresholdStd)
    int iNumTemplates = 0;
    float fThresholdStd = 3.f;
};

class SorterError : public std::runtime_error {
public:
    SorterError(int st, const std::string& m) : std::runtime_error(m), status(st) {}
    int status;
};

using SpikeSink = std::function<void(const lss_spike* spikes, int64_t n)>;

class OnlineSpikesV2 {
public:
    OnlineSpikesV2(const InputParameters& params, DataSocket* socket, SpikeSink sink = nullptr);
    ~OnlineSpikesV2();
    OnlineSpikesV2(const OnlineSpikesV2&) = delete;
    OnlineSpikesV2& operator=(const OnlineSpikesV2&) = delete;

    // The per-batch loop of OnlineSpikesV2.cu:698-849: wait for data, apply the behind/skip
    // policy, push the rows, emit finished spikes.  Returns when the socket stops running or
    // stop() was called; the buffered tail is flushed.
    void runSpikeSorting();
    void stop() { running_ = false; }

    lss_handle* handle() const { return h_; }
    int64_t skips() const { return skips_; }
    int64_t spikesWritten() const { return written_; }

private:
    void emit();
    lss_handle* h_ = nullptr;
    InputParameters params_;
    DataSocket* sock_ = nullptr;
    SpikeSink sink_;
    OSSSpecificParams os_;
    std::ofstream out_;
    std::vector<int16_t> buf_;
    std::vector<lss_spike> spikes_;
    volatile bool running_ = true;
    int64_t skips_ = 0, written_ = 0;
    int cin_ = 0;
};

}  // namespace lss
