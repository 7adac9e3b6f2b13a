// Host-only driver of lss::run_ingest_loop (include/lss_online_spikes_v2.hpp) with a scripted
// DataSocket, for tests/test_ingest_policy_cpu.py.  No GPU and no library: the loop's push and
// emit are recorded instead of sorted.
//
// stdin:  maxRows minRows timeBehindMs rateHz smallSkip first_latest
//         n_steps latest_1 ... latest_n      (stream sample count seen at each wait)
// stdout: one line per push "start n first_row_value last_row_value", then "skips K"
#include <cstdio>
#include <vector>

#include "lss_online_spikes_v2.hpp"

namespace {

class ScriptedSocket : public lss::DataSocket {
public:
    ScriptedSocket(lss::t_ull first, std::vector<lss::t_ull> script) : now_(first), script_(std::move(script)) {}
    lss::t_ull getStreamSampleCt(int, const lss::OSSSpecificParams&) override { return now_; }
    lss::t_ull fetchLatest(int16_t* data, long maxRows, const lss::OSSSpecificParams& p, lss::t_ull start) override {
        const lss::t_ull n = std::min<lss::t_ull>((lss::t_ull)maxRows, now_ - start);
        return fetchFromPlace(data, (long)n, p, now_ - n);
    }
    // rows [start, start + min(maxRows, now - start)); every value of row r is r (mod 2^15)
    lss::t_ull fetchFromPlace(int16_t* data, long maxRows, const lss::OSSSpecificParams& p, lss::t_ull start) override {
        if (start >= now_) return start;
        const lss::t_ull n = std::min<lss::t_ull>((lss::t_ull)maxRows, now_ - start);
        for (lss::t_ull r = 0; r < n; ++r)
            for (long c = 0; c < p.lNChans; ++c) data[r * p.lNChans + c] = (int16_t)((start + r) & 0x7fff);
        return start + n;
    }
    // each wait advances the acquisition to the next scripted sample count
    void waitUntil(lss::t_ull, const lss::OSSSpecificParams&) override {
        if (i_ < script_.size()) now_ = script_[i_++];
        else done_ = true;
    }
    bool isRunning() override { return !done_; }

private:
    lss::t_ull now_;
    std::vector<lss::t_ull> script_;
    size_t i_ = 0;
    bool done_ = false;
};

}  // namespace

int main() {
    long maxRows = 0, minRows = 0, behind = 0;
    double rate = 0;
    int small = 0;
    unsigned long long first = 0;
    size_t n = 0;
    if (std::scanf("%ld %ld %ld %lf %d %llu %zu", &maxRows, &minRows, &behind, &rate, &small, &first, &n) != 7)
        return 2;
    std::vector<lss::t_ull> script(n);
    for (auto& v : script)
        if (std::scanf("%llu", &v) != 1) return 2;
    lss::InputParameters prm;
    prm.iMaxScanWindow = (int)maxRows;
    prm.iMinScanWindow = (int)minRows;
    prm.iTimeBehind = (int)behind;
    prm.fImecSamplingRate = (float)rate;
    prm.bSmallskip = small != 0;
    lss::OSSSpecificParams os;
    os.lNChans = 2;
    std::vector<int16_t> buf((size_t)(maxRows + minRows) * os.lNChans);
    ScriptedSocket sock(first, script);
    bool running = true;
    int64_t skips = 0;
    lss::run_ingest_loop(
        &sock, os, prm, buf,
        [](const int16_t* rows, int64_t k, int64_t start) {
            std::printf("%lld %lld %d %d\n", (long long)start, (long long)k, rows[0], rows[(k - 1) * 2 + 1]);
        },
        []() {}, &running, &skips);
    std::printf("skips %lld\n", (long long)skips);
    return 0;
}
