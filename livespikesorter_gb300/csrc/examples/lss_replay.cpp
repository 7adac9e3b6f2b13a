// lss_replay -- drive the C++ drop-in sorter (lss::OnlineSpikesV2) from a raw int16 recording,
// the way the reference's sorter is driven by SpikeGLX through a DataSocket.
//
//   lss_replay <oss_input_dir> <recording.i16> <n_chan> <out_dir> [batch_samples] [rows_per_tick]
//   lss_replay --tc <recording.i16> <n_chan> <out_dir> <threshold_std> <calib_rows> [max_window] [rows_per_tick]
//
// The recording is [n_samples][n_chan] int16.  A replay socket makes rows_per_tick new rows
// "arrive" each time the sorter asks for the stream sample count, so the sorter sees a stream
// that grows in irregular steps; spikes land in <out_dir>/spikeOutput.txt.  With --tc the
// threshold-crossing sorter (lss::ThresholdCrossing) runs instead, its per-channel means and
// medians calibrated on the first calib_rows rows (lss_tc_calibrate); events land in
// <out_dir>/SpikeOutput_TC.txt.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "lss_online_spikes_v2.hpp"
#include "lss_threshold_crossing.hpp"

class ReplaySocket : public lss::DataSocket {
public:
    ReplaySocket(std::vector<int16_t> data, int nchan, long tick) : d_(std::move(data)), c_(nchan), tick_(tick) {
        n_ = (lss::t_ull)(d_.size() / (size_t)c_);
    }
    // the stream starts empty; every query afterwards finds rows_per_tick more rows
    lss::t_ull getStreamSampleCt(int, const lss::OSSSpecificParams&) override {
        const lss::t_ull now = avail_;
        avail_ = std::min(n_, avail_ + (lss::t_ull)tick_);
        return now;
    }
    lss::t_ull fetchLatest(int16_t* out, long maxRows, const lss::OSSSpecificParams& p, lss::t_ull start) override {
        lss::t_ull s = std::max(start, avail_ > (lss::t_ull)maxRows ? avail_ - (lss::t_ull)maxRows : 0ULL);
        return fetchFromPlace(out, maxRows, p, s);
    }
    lss::t_ull fetchFromPlace(int16_t* out, long maxRows, const lss::OSSSpecificParams&, lss::t_ull start) override {
        lss::t_ull end = std::min(avail_, start + (lss::t_ull)maxRows);
        if (end <= start) return start;
        std::copy(d_.begin() + (long)(start * c_), d_.begin() + (long)(end * c_), out);
        fetched_ = std::max(fetched_, end);
        return end;
    }
    bool isRunning() override { return fetched_ < n_; }
    void waitUntil(lss::t_ull, const lss::OSSSpecificParams&) override {}

private:
    std::vector<int16_t> d_;
    int c_;
    long tick_;
    lss::t_ull n_ = 0, avail_ = 0, fetched_ = 0;
};

static bool read_i16(const char* path, std::vector<int16_t>& data) {
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f) return false;
    const std::streamsize bytes = f.tellg();
    f.seekg(0);
    data.resize((size_t)bytes / 2);
    f.read(reinterpret_cast<char*>(data.data()), bytes);
    return (bool)f;
}

static int run_tc(int argc, char** argv) {
    if (argc < 7) {
        std::fprintf(stderr, "usage: %s --tc recording.i16 n_chan out_dir threshold_std calib_rows [max_window] [rows_per_tick]\n",
                     argv[0]);
        return 2;
    }
    const int nchan = std::atoi(argv[3]);
    std::vector<int16_t> data;
    if (nchan < 1 || !read_i16(argv[2], data)) {
        std::fprintf(stderr, "cannot read %s\n", argv[2]);
        return 2;
    }
    const long nrows = (long)(data.size() / (size_t)nchan);
    const long calib = std::min<long>(std::atol(argv[6]), nrows);
    std::vector<float> means(nchan), medians(nchan);
    if (calib < 1 || lss_tc_calibrate(data.data(), calib, nchan, means.data(), medians.data()) != LSS_OK) {
        std::fprintf(stderr, "calibration failed\n");
        return 2;
    }
    lss::InputParameters ip;
    ip.sOSSOutputFolder = argv[4];
    ip.iNumTemplates = nchan;
    ip.fThresholdStd = (float)std::atof(argv[5]);
    if (argc > 7) ip.iMaxScanWindow = std::atoi(argv[7]);
    const long tick = argc > 8 ? std::atol(argv[8]) : 977;
    try {
        ReplaySocket sock(std::move(data), nchan, tick);
        lss::ThresholdCrossing tc(ip, means, medians, &sock);
        tc.runThresholdCrossing();
        std::printf("events %lld\n", (long long)tc.eventsWritten());
    } catch (const lss::SorterError& e) {
        std::fprintf(stderr, "error %d: %s\n", e.status, e.what());
        return 1;
    }
    return 0;
}

int main(int argc, char** argv) {
    if (argc > 1 && std::string(argv[1]) == "--tc") return run_tc(argc, argv);
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s oss_dir recording.i16 n_chan out_dir [batch_samples] [rows_per_tick]\n", argv[0]);
        return 2;
    }
    const int nchan = std::atoi(argv[3]);
    std::vector<int16_t> data;
    if (!read_i16(argv[2], data)) {
        std::fprintf(stderr, "cannot open %s\n", argv[2]);
        return 2;
    }
    lss::InputParameters ip;
    ip.sInputFolder = argv[1];
    ip.sOSSOutputFolder = argv[4];
    if (argc > 5) ip.iMaxScanWindow = std::atoi(argv[5]);
    const long tick = argc > 6 ? std::atol(argv[6]) : 977;
    ip.iTimeBehind = 100000;   // replay: never skip
    ip.iMaxIts = 100;
    try {
        ReplaySocket sock(std::move(data), nchan, tick);
        lss::OnlineSpikesV2 sorter(ip, &sock);
        sorter.runSpikeSorting();
        std::printf("spikes %lld skips %lld\n", (long long)sorter.spikesWritten(), (long long)sorter.skips());
    } catch (const lss::SorterError& e) {
        std::fprintf(stderr, "error %d: %s\n", e.status, e.what());
        return 1;
    }
    return 0;
}
