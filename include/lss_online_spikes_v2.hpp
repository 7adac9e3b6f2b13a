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

// Where the next fetch starts: the behind/skip policy of OnlineSpikesV2::runSpikeSorting
// (OnlineSpikesV2.cu:705-746), one branch per case.
enum class FetchBranch {
    Normal,      // at most one batch behind: the rows after the last processed one (:712-719)
    JumpNewest,  // behind, and being behind is not allowed (iTimeBehind == 0): the newest batch (:720-724)
    CatchUp,     // behind, but within iTimeBehind ms: keep going from the last processed row (:728-732)
    SmallSkip,   // further behind than allowed, bSmallskip: from the newest row allowed (:734-738)
    BigSkip      // further behind than allowed, no small skip: the newest batch (:740-746)
};

struct FetchPlan {
    t_ull start;        // stream sample of the first row to fetch
    bool skip;          // rows between the last processed one and start are dropped
    FetchBranch branch;
};

// The reference computes allowedCt = latestCt - timeBehind * samplingRate / 1000 in float
// (OnlineSpikesV2.cu:707), which rounds sample counts above 2^24; here the allowed lag is an exact
// sample count and allowedCt never goes below 0.
inline FetchPlan plan_fetch(t_ull latest, t_ull processed, long maxRows, long timeBehindMs, double rateHz,
                            bool smallSkip) {
    const t_ull lag = timeBehindMs > 0 ? (t_ull)((double)timeBehindMs * rateHz / 1000.0) : 0;
    const t_ull allowedCt = latest > lag ? latest - lag : 0;
    const t_ull newest = latest > (t_ull)maxRows ? latest - (t_ull)maxRows : 0;
    if (latest - processed <= (t_ull)maxRows) return {processed, false, FetchBranch::Normal};
    if (timeBehindMs == 0) return {newest, true, FetchBranch::JumpNewest};
    if (processed >= allowedCt) return {processed, false, FetchBranch::CatchUp};
    if (smallSkip) return {allowedCt, true, FetchBranch::SmallSkip};
    return {newest, true, FetchBranch::BigSkip};
}

// The acquisition loop of runSpikeSorting (OnlineSpikesV2.cu:698-849) over any DataSocket: wait for
// iMinScanWindow new rows, plan the fetch, fetch up to iMaxScanWindow rows from the planned start,
// hand them to push(rows, n, first_stream_sample), then emit().  Returns when the socket stops
// running or *running turns false.  Counts skips in *skips.  Header-only so that the policy can be
// driven without a GPU.
template <typename Push, typename Emit>
void run_ingest_loop(DataSocket* sock, const OSSSpecificParams& os, const InputParameters& prm,
                     std::vector<int16_t>& buf, Push&& push, Emit&& emit, const volatile bool* running,
                     int64_t* skips) {
    const long maxRows = prm.iMaxScanWindow;
    t_ull latest = sock->getStreamSampleCt(IMEC, os);
    t_ull processed = latest;
    while (*running && sock->isRunning()) {
        sock->waitUntil(processed + (t_ull)prm.iMinScanWindow, os);
        latest = sock->getStreamSampleCt(IMEC, os);
        if (latest <= processed) {
            if (!sock->isRunning()) break;
            continue;
        }
        const FetchPlan fp = plan_fetch(latest, processed, maxRows, prm.iTimeBehind, prm.fImecSamplingRate,
                                        prm.bSmallskip);
        if (fp.skip) ++*skips;
        const t_ull end = sock->fetchFromPlace(buf.data(), maxRows, os, fp.start);
        if (end <= fp.start) continue;
        push(buf.data(), (int64_t)(end - fp.start), (int64_t)fp.start);
        processed = end;
        emit();
    }
}

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
