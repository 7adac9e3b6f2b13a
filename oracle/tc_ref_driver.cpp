// tc_ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.  Runs the reference's ThresholdCrossing class
// (src/SpikeSorter/ThresholdCrossing.cpp, compiled unmodified with tc_ref_stubs.h force-included)
// on a scripted replay of int16 rows, to produce golden threshold-crossing events.
//
//   tc_ref ROWS.bin C SCHEDULE... 
// ROWS.bin: int16 [N][C] (channel fastest), row s = stream sample s.  SCHEDULE: the stream sample
// counts the replay socket reports, one per wait (the first is the count at start).  The run ends
// when the schedule is exhausted.  Output: one line per sent payload, "latest n_events" followed by
// that many "time,channel" lines, in the order the reference emits them.
#include "ThresholdCrossing.h"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>

namespace {
std::vector<int16_t> g_rows;
long g_C = 0;
std::vector<long> g_sched;
size_t g_at = 0;
struct EndOfScript {};
std::vector<OnlineSpikesPayload> g_sent;
}  // namespace

void record_payload(const OnlineSpikesPayload& p) { g_sent.push_back(p); }

StreamDataSocket::StreamDataSocket(std::string, uint16, int, long lMaxSize, long lMinSize, float, float, int)
    : m_lMaxSize(lMaxSize), m_lMinSize(lMinSize) {}

t_ull StreamDataSocket::getStreamSampleCt(int, OSSSpecificParams) { return (t_ull)g_sched[g_at]; }

// rows [start, latest) as the reference's StreamDataSocket::fetchLatest_TC chooses them
// (dataSocket.cpp:128-153): the default start fetches the minimum window, at most the maximum
// window is fetched (the newest rows); returns the row count
t_ull StreamDataSocket::fetchLatest_TC(float* fData, OSSSpecificParams osParams, t_ull lStartCt) {
    const t_ull latest = getStreamSampleCt(IMEC, osParams);
    t_ull toGet = latest - lStartCt;
    if (lStartCt == ULLONG_MAX) {
        toGet = (t_ull)m_lMinSize;
        lStartCt = latest - m_lMinSize;
    }
    if (toGet > (t_ull)m_lMaxSize) {
        toGet = (t_ull)m_lMaxSize;
        lStartCt = latest - m_lMaxSize;
    }
    for (t_ull r = 0; r < toGet; ++r)
        for (long c = 0; c < osParams.lNChans; ++c)
            fData[r * osParams.lNChans + c] = (float)g_rows[(size_t)(lStartCt + r) * g_C + osParams.vImecChannels[c]];
    return toGet;
}

void StreamDataSocket::waitUntil(t_ull lCt, OSSSpecificParams) {
    while ((t_ull)g_sched[g_at] < lCt) {
        if (++g_at >= g_sched.size()) throw EndOfScript{};
    }
}

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: tc_ref ROWS.bin C MIN MAX THRESHOLD_STD SCHEDULE...\n");
        return 2;
    }
    std::ifstream f(argv[1], std::ios::binary | std::ios::ate);
    const std::streamsize bytes = f.tellg();
    f.seekg(0);
    g_rows.resize((size_t)bytes / 2);
    f.read(reinterpret_cast<char*>(g_rows.data()), bytes);
    g_C = std::atol(argv[2]);
    InputParameters p;
    p.iMinScanWindow = std::atoi(argv[3]);
    p.iMaxScanWindow = std::atoi(argv[4]);
    p.fThresholdStd = (float)std::atof(argv[5]);
    p.iNumTemplates = (int)g_C;
    for (int i = 6; i < argc; ++i) g_sched.push_back(std::atol(argv[i]));
    std::streambuf* keep = std::cout.rdbuf();
    std::ofstream devnull("/dev/null");
    std::cout.rdbuf(devnull.rdbuf());   // the class's progress prints
    DataSocket* sock = nullptr;
    DataSocket** ps = &sock;
    ThresholdCrossing tc(p, sockaddr_in{}, ps);
    try {
        tc.runThresholdCrossing();
    } catch (const EndOfScript&) {
    }
    std::cout.rdbuf(keep);
    for (const OnlineSpikesPayload& q : g_sent) {
        std::printf("%ld %zu\n", q.streamSampleCt, q.Times.size());
        for (size_t i = 0; i < q.Times.size(); ++i) std::printf("%ld,%ld\n", q.Times[i], q.Templates[i]);
    }
    return 0;
}
