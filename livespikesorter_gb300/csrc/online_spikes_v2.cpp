// online_spikes_v2.cpp -- the C++ drop-in sorter class over the C ABI (see
// include/lss_online_spikes_v2.hpp).
#include "../../include/lss_online_spikes_v2.hpp"

#include <algorithm>
#include <cstdio>
#include <filesystem>

namespace lss {

static void check(lss_handle* h, int st) {
    if (st != LSS_OK) throw SorterError(st, lss_last_error(h));
}

OnlineSpikesV2::OnlineSpikesV2(const InputParameters& params, DataSocket* socket, SpikeSink sink)
    : params_(params), sock_(socket), sink_(std::move(sink)) {
    if (!sock_) throw SorterError(LSS_ERR_ARG, "OnlineSpikesV2: null DataSocket");
    lss_params p;
    lss_default_params(&p);
    p.device = params.uSelectedDevice;
    p.batch_samples = params.iMaxScanWindow;
    p.max_iters = params.iMaxIts;
    p.group_batches = params.iGroupBatches;
    p.n_chan_in = params.iChannelsIn;
    const int st = lss_open(params.sInputFolder.c_str(), &p, &h_);
    if (st != LSS_OK) throw SorterError(st, lss_last_error(nullptr));
    lss_info info;
    lss_get_info(h_, &info);
    cin_ = params.iChannelsIn > 0 ? params.iChannelsIn : info.C;
    os_.lNChans = cin_;
    os_.substream = params.iSubstream;
    os_.vImecChannels.resize(cin_);
    for (int c = 0; c < cin_; ++c) os_.vImecChannels[c] = c;
    if (!params.sOSSOutputFolder.empty()) {
        // keep an earlier output file, like OnlineSpikesV2.cu:333-352
        namespace fs = std::filesystem;
        fs::create_directories(params.sOSSOutputFolder);
        fs::path f = fs::path(params.sOSSOutputFolder) / "spikeOutput.txt";
        if (fs::exists(f)) {
            int k = 1;
            fs::path r;
            do {
                r = fs::path(params.sOSSOutputFolder) / ("spikeOutput_" + std::to_string(k++) + ".txt");
            } while (fs::exists(r));
            fs::rename(f, r);
        }
        out_.open(f);
        if (!out_) throw SorterError(LSS_ERR_IO, "cannot open " + f.string());
    }
    buf_.resize((size_t)(params.iMaxScanWindow + params.iMinScanWindow) * cin_);
    spikes_.resize(1 << 14);
}

OnlineSpikesV2::~OnlineSpikesV2() {
    if (h_) lss_close(h_);
}

void OnlineSpikesV2::emit() {
    for (;;) {
        int64_t n = 0;
        const int st = lss_poll(h_, spikes_.data(), (int64_t)spikes_.size(), &n);
        if (st != LSS_OK && st != LSS_ERR_OVERFLOW) check(h_, st);
        if (n > 0) {
            if (out_.is_open()) {
                for (int64_t i = 0; i < n; ++i)
                    out_ << spikes_[i].time << "," << spikes_[i].cluster << "," << spikes_[i].amp << ","
                         << spikes_[i].y << "\n";
                out_.flush();
            }
            if (sink_) sink_(spikes_.data(), n);
            written_ += n;
        }
        if (n < (int64_t)spikes_.size()) break;
    }
}

void OnlineSpikesV2::runSpikeSorting() {
    // a fetch that starts after the previous one's end (a skip) is a discontinuity: lss_push_batch
    // flushes the segment and starts a new one there
    run_ingest_loop(
        sock_, os_, params_, buf_,
        [this](const int16_t* rows, int64_t n, int64_t start) { check(h_, lss_push_batch(h_, rows, n, start)); },
        [this]() { emit(); }, &running_, &skips_);
    check(h_, lss_flush(h_));
    int64_t pend = 0;
    check(h_, lss_pending(h_, &pend));
    emit();
}

}  // namespace lss
