// lss_noalloc.cu -- the matching loop on caller-owned buffers, with no memory allocation.
//
// Some callers cannot allocate device memory at the point where they sort: a real-time
// acquisition thread that must not block on the allocator, code that runs inside a fixed
// memory pool owned by another framework, or an application that already holds the scores
// and residual in its own buffers.  lss_match_noalloc runs the same matching-pursuit kernel as
// the rest of the library, but its working memory (the per-sample maxima of long windows and the
// accepted-spike maps) lives in the statically sized device array below instead of buffers
// obtained from cudaMalloc.
//
// The array is a file-scope __device__ variable: every GPU that loads this library holds it
// (LSS_NOALLOC_SCRATCH_BYTES) until the process exits.  Host code cannot use its name as a
// device address, so each call made outside stream capture looks the address up with
// cudaGetSymbolAddress (with the caller's device current) and keeps it per device; a call made
// while its stream is being captured uses the kept address, so the first call on a device must
// come before any capture.  Looking the address up again on every uncaptured call keeps it valid
// after cudaDeviceReset, which reloads the module at a new address.  Every call shares the one
// array and it keeps the previous call's contents, so the parts that must start at zero are
// cleared on the caller's stream at each call; calls whose kernels overlap on the GPU race on the
// array.  The kernel's status word also lives there; a small kernel after the loop turns a fault
// it reports into a negative *n_spikes, so no host read of the array is needed.
#include "../../include/lss_gb300.h"
#include "lss_kernels.cuh"

#include <mutex>
#include <string>

namespace lss {
extern thread_local std::string g_handleless_error;
}

namespace {

constexpr int kMaxW = LSS_NOALLOC_MAX_SAMPLES;
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t n) { return (n + kAlign - 1) / kAlign * kAlign; }
// layout of the scratch array (byte offsets)
constexpr size_t kOffCfmax = 0;
constexpr size_t kOffAtT = align_up(kOffCfmax + sizeof(float) * kMaxW);
constexpr size_t kOffAtAmp = align_up(kOffAtT + sizeof(int) * kMaxW);
constexpr size_t kOffStatus = align_up(kOffAtAmp + sizeof(float) * kMaxW);
constexpr size_t kOffIters = kOffStatus + sizeof(int);
constexpr size_t kScratchBytes = align_up(kOffIters + sizeof(int));
static_assert(kScratchBytes == LSS_NOALLOC_SCRATCH_BYTES, "scratch size in lss_gb300.h is out of date");

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {};

// status bit 0 (more spikes than cap) is visible as *n_spikes > cap already; any other bit means
// the loop did not run as launched and its lists are not valid: report -(those bits)
__global__ void noalloc_status_kernel(const int* status, int* n_spikes) {
    const int bad = *status & ~1;
    if (bad) *n_spikes = -bad;
}

}  // namespace

extern "C" int lss_match_noalloc(float* scores, float* residual, const float* ctc_perm, const float* waveforms,
                                 const float* template_norms, float th, int32_t W, int32_t T, int32_t C, int32_t nt,
                                 int32_t max_iters, int32_t* n_spikes, int32_t* spike_sample,
                                 int32_t* spike_template, float* spike_amp, int32_t* spike_iter, int32_t cap,
                                 void* stream) {
    std::string& g_noalloc_error = lss::g_handleless_error;
    if (!scores || !residual || !ctc_perm || !waveforms || !template_norms || !n_spikes || cap < 0 ||
        (cap > 0 && (!spike_sample || !spike_template || !spike_amp || !spike_iter))) {
        g_noalloc_error = "lss_match_noalloc: null pointer or negative cap";
        return LSS_ERR_ARG;
    }
    if (W > kMaxW) {
        g_noalloc_error = "lss_match_noalloc: window of " + std::to_string(W) + " samples exceeds the maximum of " +
                          std::to_string(kMaxW) + " (LSS_NOALLOC_MAX_SAMPLES)";
        return LSS_ERR_ARG;
    }
    if (W <= 2 * nt + 1 || T <= 0 || C <= 0 || nt <= 0 || nt % 2 == 0 || max_iters <= 0 || !(th > 0.f)) {
        g_noalloc_error = "lss_match_noalloc: bad W / T / C / nt / max_iters / th";
        return LSS_ERR_ARG;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        g_noalloc_error = std::string("lss_match_noalloc: cudaGetDevice: ") + cudaGetErrorString(e);
        return LSS_ERR_CUDA;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap_st = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(s, &cap_st);
    if (e != cudaSuccess) {
        g_noalloc_error = std::string("lss_match_noalloc: cudaStreamIsCapturing: ") + cudaGetErrorString(e);
        return LSS_ERR_CUDA;
    }
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (cap_st == cudaStreamCaptureStatusNone) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_scratch);   // the current device is dev
            if (e != cudaSuccess) {
                g_noalloc_error = std::string("lss_match_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
                return LSS_ERR_CUDA;
            }
            g_addr[dev] = static_cast<unsigned char*>(p);
        } else if (!g_addr[dev]) {
            g_noalloc_error = "lss_match_noalloc: the first call on a device must come before stream capture";
            return LSS_ERR_ARG;
        }
        base = g_addr[dev];
    }
    lss::MatchScratch sc{};
    sc.cfmax = reinterpret_cast<float*>(base + kOffCfmax);
    sc.at_t = reinterpret_cast<int*>(base + kOffAtT);
    sc.at_amp = reinterpret_cast<float*>(base + kOffAtAmp);
    lss::MatchOut out{};
    out.n_spikes = n_spikes;
    out.n_iters = reinterpret_cast<int*>(base + kOffIters);
    out.status = reinterpret_cast<int*>(base + kOffStatus);
    out.sp_w = spike_sample;
    out.sp_t = spike_template;
    out.sp_amp = spike_amp;
    out.sp_iter = spike_iter;
    out.cap = cap;
    // the status word is accumulated with atomicOr: it must start at zero on every call
    e = cudaMemsetAsync(out.status, 0, sizeof(int), s);
    if (e == cudaSuccess)
        e = lss::launch_match(scores, residual, ctc_perm, waveforms, template_norms, th * th, W, T, C, nt, max_iters,
                              1, sc, out, s, 0);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) {
        noalloc_status_kernel<<<1, 1, 0, s>>>(out.status, n_spikes);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        g_noalloc_error = std::string("lss_match_noalloc: ") + cudaGetErrorString(e);
        return LSS_ERR_CUDA;
    }
    return LSS_OK;
}
