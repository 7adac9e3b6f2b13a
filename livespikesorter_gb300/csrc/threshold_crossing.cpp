// threshold_crossing.cpp -- the C++ drop-in threshold-crossing sorter over the C ABI of
// lss_threshold.h (class declared in include/lss_threshold_crossing.hpp).
#include "../../include/lss_threshold_crossing.hpp"

#include <algorithm>
#include <filesystem>
#include <string>

namespace lss {

ThresholdCrossing::ThresholdCrossing(const InputParameters& params, const std::vector<float>& means,
                                     const std::vector<float>& medians, DataSocket* socket, EventSink sink)
    : params_(params), sock_(socket), sink_(std::move(sink)), c_(params.iNumTemplates) {
    if (!sock_) throw SorterError(LSS_ERR_ARG, "ThresholdCrossing: null DataSocket");
    if (c_ < 1 || (int)means.size() != c_ || (int)medians.size() != c_)
        throw SorterError(LSS_ERR_ARG, "ThresholdCrossing: need iNumTemplates channels of means and medians");
    if (params.iMaxScanWindow < 1 || params.iMinScanWindow < 0)
        throw SorterError(LSS_ERR_ARG, "ThresholdCrossing: bad scan windows");
    lss_tc_params p;
    lss_tc_default_params(&p);
    p.device = params.uSelectedDevice;
    p.n_chan = c_;
    p.threshold_std = params.fThresholdStd;
    p.max_rows = params.iMaxScanWindow;
    const int st = lss_tc_open(&p, means.data(), medians.data(), &h_);
    if (st != LSS_OK) throw SorterError(st, lss_tc_last_error(nullptr));
    os_.lNChans = c_;
    os_.substream = 0;   // the reference never parallelises this sorter (ThresholdCrossing.cpp:118)
    os_.vImecChannels.resize(c_);
    for (int c = 0; c < c_; ++c) os_.vImecChannels[c] = c;
    if (!params.sOSSOutputFolder.empty()) {
        namespace fs = std::filesystem;
        fs::create_directories(params.sOSSOutputFolder);
        const fs::path f = fs::path(params.sOSSOutputFolder) / "SpikeOutput_TC.txt";
        out_ = std::fopen(f.string().c_str(), "w");
        if (!out_) {
            lss_tc_close(h_);
            h_ = nullptr;
            throw SorterError(LSS_ERR_IO, "cannot open " + f.string());
        }
    }
    buf_.resize((size_t)params.iMaxScanWindow * c_);
    ev_.resize(1 << 14);
}

ThresholdCrossing::~ThresholdCrossing() {
    if (out_) std::fclose(out_);
    if (h_) lss_tc_close(h_);
}

void ThresholdCrossing::emit() {
    for (;;) {
        int64_t n = 0;
        const int st = lss_tc_poll(h_, ev_.data(), (int64_t)ev_.size(), &n);
        if (st != LSS_OK && st != LSS_ERR_OVERFLOW) throw SorterError(st, lss_tc_last_error(h_));
        if (n == 0) break;
        if (out_)
            for (int64_t i = 0; i < n; ++i)
                std::fprintf(out_, "%20ld,%4ld,%f\n", (long)ev_[i].time, (long)ev_[i].channel, 0.0);
        if (sink_) sink_(ev_.data(), n);
        written_ += n;
        if (n < (int64_t)ev_.size()) break;
    }
    if (out_) std::fflush(out_);
}

void ThresholdCrossing::runThresholdCrossing() {
    t_ull processed = sock_->getStreamSampleCt(IMEC, os_);
    while (running_) {
        sock_->waitUntil(processed + (t_ull)params_.iMinScanWindow, os_);
        const t_ull latest = sock_->getStreamSampleCt(IMEC, os_);
        if (latest <= processed) {
            if (!sock_->isRunning()) break;
            continue;
        }
        // rows [processed, latest), the newest iMaxScanWindow when more arrived
        // (StreamDataSocket::fetchLatest_TC, dataSocket.cpp:128-154)
        const t_ull end = sock_->fetchLatest(buf_.data(), params_.iMaxScanWindow, os_, processed);
        if (end <= processed) {
            if (!sock_->isRunning()) break;
            continue;
        }
        const int64_t n = (int64_t)std::min<t_ull>(end - processed, (t_ull)params_.iMaxScanWindow);
        const int st = lss_tc_push(h_, buf_.data(), n, (int64_t)(end - (t_ull)n));
        if (st != LSS_OK) throw SorterError(st, lss_tc_last_error(h_));
        emit();
        processed = end;
    }
    emit();
}

}  // namespace lss
