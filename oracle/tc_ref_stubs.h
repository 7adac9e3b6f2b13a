// tc_ref_stubs.h -- TEST INFRASTRUCTURE ONLY.  Force-included (g++ -include) ahead of the
// reference's src/SpikeSorter/ThresholdCrossing.cpp so that file compiles unmodified on Linux
// without Winsock, the SpikeGLX SDK or the reference's networking layer: it defines the include
// guards of the headers ThresholdCrossing.cpp / ThresholdCrossing.h pull in (Helpers/Utils.h,
// SpikeSorter/dataSocket.h, Networking/{inputParameters,Sock,sorterParameters,FragmentManager,
// onlineSpikesPayload,NetworkHelpers}.h) and declares in their place the few types and calls
// that code uses.  The data socket is a scripted replay (tc_ref_driver.cpp); sending a payload
// records it.  Nothing of the reference's own logic is restated here.
#pragma once
#define UTILS_H_
#define DATA_SOCKET_H_
#define INPUTPARAMETERS_H
#define SOCK_H
#define SORTPARAMETERS_H
#define FRAGMENT_MANAGER_H
#define ONLINESPIKESPAYLOAD_H
#define NETWORKHELPERS_H

#include <netinet/in.h>
#include <climits>
#include <cstdint>
#include <ctime>
#include <string>
#include <thread>
#include <vector>

typedef unsigned long long t_ull;
typedef unsigned short uint16;
enum streamTypes { NIDQ, OBX, IMEC };
struct t_sglxconn {};

struct OSSSpecificParams {
    long lNChans;
    std::vector<int> vImecChannels;
    int substream;
};

class DataSocket {
public:
    virtual ~DataSocket() {}
    virtual t_ull getStreamSampleCt(int streamType, OSSSpecificParams osParams) = 0;
    virtual t_ull fetchLatest_TC(float* fData, OSSSpecificParams osParams, t_ull lStartCt = ULLONG_MAX) = 0;
    virtual bool startRun() { return true; }
    virtual void waitUntil(t_ull lCt, OSSSpecificParams osParams) = 0;
};

// the replay socket (defined in tc_ref_driver.cpp)
class StreamDataSocket : public DataSocket {
public:
    StreamDataSocket(std::string host, uint16 port, int substream, long lMaxSize, long lMinSize, float fImecSampRate,
                     float fNidqSampRate, int downSampling);
    t_ull getStreamSampleCt(int streamType, OSSSpecificParams osParams) override;
    t_ull fetchLatest_TC(float* fData, OSSSpecificParams osParams, t_ull lStartCt = ULLONG_MAX) override;
    void waitUntil(t_ull lCt, OSSSpecificParams osParams) override;

private:
    long m_lMaxSize, m_lMinSize;
};

struct InputParameters {
    std::string sDataAccquisitionHost;
    uint16 uDataAccquisitionPort = 0;
    float fImecSamplingRate = 30000.f, fNidqSamplingRate = 0.f, fThresholdStd = 0.f;
    int iSubstream = 0, iMinScanWindow = 0, iMaxScanWindow = 0, iDownsampling = 1, iNumTemplates = 0;
};

class Sock {
public:
    enum Type { UDP, TCP };
    explicit Sock(Type) {}
};

class FragmentManager {
public:
    explicit FragmentManager(Sock*) {}
    std::thread assemblerThread() { return std::thread([] {}); }
    std::thread retransmitterThread() { return std::thread([] {}); }
};

struct SorterParameters {
    long m_lT, m_lC, m_lM, m_lN;
    float m_fSampRate;
    std::vector<double> m_dChanpos;
};

struct OnlineSpikesPayload {
    long recordingOffset;
    long streamSampleCt;
    std::vector<long> Times;
    std::vector<long> Templates;
    std::vector<float> Amplitudes;
    double VRMS;
    float P2P;
    long processTime;
};

#define _SPIKE_SORTER_IMEC 0
#define _SPIKE_SORTER_NIDQ 1
#define _DECODER_IMEC 2
#define _DECODER_NIDQ 3
inline void sendConnectMsg(Sock*, sockaddr_in, uint16) {}
inline sockaddr_in recvConnectMsg(Sock*, uint16) { return sockaddr_in{}; }
void record_payload(const OnlineSpikesPayload& p);   // tc_ref_driver.cpp
inline void sendPayload(FragmentManager*, const SorterParameters&, const sockaddr_in&) {}
inline void sendPayload(FragmentManager*, const OnlineSpikesPayload& p, const sockaddr_in&) { record_payload(p); }
inline int clock_gettime(timespec& t) {
    t = timespec{};
    return 0;
}
inline int GetTimeDiff(timespec, timespec) { return 0; }
