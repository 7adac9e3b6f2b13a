// sorter.cu -- host side of one sorter handle: device-resident state, stream framing,
// launch sequence of a group of batches, egress, and the C ABI of include/lss_gb300.h.
//
// Stream framing follows Kilosort's batching (io.py:584-637, template_matching.py:56-68): batch j
// of a segment covers the new samples [s0 + j*NT, s0 + (j+1)*NT) and is sorted on the window
// [s0 + j*NT - nt, s0 + (j+1)*NT + nt); the first window's left pad repeats the first sample, the
// last window's right side repeats the last sample.  Detections are limited to the interior of a
// window (Cf is zeroed on nt samples at both ends), so consecutive windows tile the stream
// without double counting.  The reference's own loop overlaps windows by lookback = 2M samples
// (OnlineSpikesV2.cu:844) -- the same 2*nt overlap -- and computes the spike time as
// start + s - M/2 - M + nt0min - lookback (OnlineSpikesV2.cu:1186-1187) for its framing; here the
// time is window_start + s - nt//2 + nt0min, Kilosort's formula.
#include "../../include/lss_gb300.h"
#include "../../include/lss_proposal.h"
#include "lss_kernels.cuh"
#include "oss_input.hpp"
#include "proposal.hpp"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <string>
#include <vector>

namespace lss {

struct CudaError {
    std::string msg;
};

#define LSS_CUDA(call)                                                                             \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            throw ::lss::CudaError{std::string(#call) + ": " + cudaGetErrorString(e_) + " (" +            \
                            std::to_string((int)e_) + ")"};                                        \
    } while (0)

template <typename T>
static T* dev_alloc(size_t n, int64_t& tally) {
    void* p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc(&p, n * sizeof(T));
    if (e != cudaSuccess) throw LoadError{LSS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
    tally += (int64_t)(n * sizeof(T));
    return static_cast<T*>(p);
}

template <typename T>
static T* dev_upload(const std::vector<T>& v, int64_t& tally, cudaStream_t s) {
    T* p = dev_alloc<T>(v.size(), tally);
    LSS_CUDA(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return p;
}

namespace {
// Host copies of a few hundred kB to a few MB (one batch of pageable rows into the pinned staging)
// go through a small process-wide pool of copy helpers: the copy is cut into chunks that the
// calling thread and the helpers claim from a shared counter, so a call never waits for a busy
// pool -- the caller copies whatever the helpers have not taken -- and only for chunks already
// being copied.
struct CopyJob {
    char* dst;
    const char* src;
    size_t bytes, chunk, nchunks;
    std::atomic<size_t> next{0}, done{0};
};

void copy_chunks(CopyJob& j) {
    for (size_t c; (c = j.next.fetch_add(1, std::memory_order_relaxed)) < j.nchunks;) {
        const size_t off = c * j.chunk;
        std::memcpy(j.dst + off, j.src + off, std::min(j.chunk, j.bytes - off));
        j.done.fetch_add(1, std::memory_order_release);
    }
}

class CopyPool {
  public:
    static CopyPool& get() {
        static CopyPool pool;
        return pool;
    }
    size_t helpers() const { return th_.size(); }
    void run(void* dst, const void* src, size_t bytes, size_t chunk) {
        auto j = std::make_shared<CopyJob>();
        j->dst = static_cast<char*>(dst);
        j->src = static_cast<const char*>(src);
        j->bytes = bytes;
        j->chunk = chunk;
        j->nchunks = (bytes + chunk - 1) / chunk;
        {
            std::lock_guard<std::mutex> lk(mu_);
            q_.push_back(j);
        }
        cv_.notify_all();
        copy_chunks(*j);
        {
            std::lock_guard<std::mutex> lk(mu_);
            auto it = std::find(q_.begin(), q_.end(), j);
            if (it != q_.end()) q_.erase(it);
        }
        // chunks a helper claimed are a memcpy each from being done
        while (j->done.load(std::memory_order_acquire) < j->nchunks) std::this_thread::yield();
    }

  private:
    CopyPool() {
        const unsigned hw = std::thread::hardware_concurrency();
        const unsigned n = std::min(4u, hw / 4);
        for (unsigned i = 0; i < n; ++i) th_.emplace_back([this] { work(); });
    }
    ~CopyPool() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : th_) t.join();
    }
    void work() {
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            cv_.wait(lk, [this] { return stop_ || !q_.empty(); });
            if (stop_) return;
            std::shared_ptr<CopyJob> j = q_.front();
            lk.unlock();
            copy_chunks(*j);
            lk.lock();
            if (!q_.empty() && q_.front() == j) q_.pop_front();   // every chunk is claimed
        }
    }
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<std::shared_ptr<CopyJob>> q_;
    bool stop_ = false;
    std::vector<std::thread> th_;
};
}  // namespace

// memcpy split across threads for large host copies (pinned staging fills at several GB/s per
// core; one thread alone is the bottleneck of the host path): copies of 8 MB and more on threads
// of their own, from 512 kB on the copy pool
void par_memcpy(void* dst, const void* src, size_t bytes) {
    constexpr size_t kChunk = 4u << 20;
    constexpr size_t kPoolMin = 512u << 10, kPoolChunk = 256u << 10;
    const size_t nthr = std::min<size_t>(std::max(1u, std::thread::hardware_concurrency() / 2), 16);
    if (bytes < 2 * kChunk) {
        if (bytes >= kPoolMin && CopyPool::get().helpers() > 0) {
            CopyPool::get().run(dst, src, bytes, kPoolChunk);
            return;
        }
        std::memcpy(dst, src, bytes);
        return;
    }
    if (nthr < 2) {
        std::memcpy(dst, src, bytes);
        return;
    }
    const size_t k = std::min(nthr, bytes / kChunk);
    const size_t per = ((bytes + k - 1) / k + 63) / 64 * 64;   // k * per >= bytes: nothing left over
    std::vector<std::thread> th;
    th.reserve(k);
    for (size_t i = 1; i < k; ++i) {
        const size_t off = i * per;
        if (off >= bytes) break;
        const size_t n = std::min(per, bytes - off);
        th.emplace_back([=] { std::memcpy((char*)dst + off, (const char*)src + off, n); });
    }
    std::memcpy(dst, src, std::min(per, bytes));
    for (auto& t : th) t.join();
}

struct TapSet {
    float* d = nullptr;          // taps, zero-padded to a multiple of 32 (SIMT FIR)
    int L = 0, R = 0;
    // tensor-core high-pass, for the small [0] and large [1] output tiles: the tile x Kt band
    // matrix G[j][k] = taps[k - j] (tf32 split) and the tensor maps over the channel-major window
    // buffer, whose row pitch is `pitch`
    float *g_hi[2] = {}, *g_lo[2] = {};
    int Kt[2] = {};
    int pitch = 0;
    UmmaOperands* um[2] = {};
    // tensor-core basis convolution: maps over the channel-major whitened windows (row pitch
    // zpitch = W rounded up to 8) and the band tiles
    int zpitch = 0;
    ConvOperands* conv = nullptr;
};
constexpr int kHighpassTile[2] = {kHighpassTileSmall, kHighpassTileLarge};

constexpr int kSlots = 4;   // groups in flight + the one collecting the stream's next rows
// the projection of a launch of at most kSplitBatches windows (26 CTAs for one 1622-sample window)
// splits K kSplitK ways to fill the GPU
constexpr int kSplitBatches = 2, kSplitK = 4;

struct Slot {
    int16_t* h_stage = nullptr;
    size_t stage_rows = 0;
    size_t recs_n = 0;          // SpikeRec capacity of h_recs
    SpikeRec* h_recs = nullptr;
    SpikeRec* d_recs = nullptr;
    int* h_off = nullptr;
    int* d_off = nullptr;
    int* h_nsp = nullptr;     // [nbcap] spikes found (may exceed cap)
    int* h_status = nullptr;  // [nbcap]
    cudaEvent_t ev = nullptr;
    cudaEvent_t ev_copy = nullptr;            // its rows are on the device (copy stream)
    cudaEvent_t tev[LSS_N_STAGES + 1] = {};   // stage boundaries (profile = 1)
    bool busy = false;
    bool reserved = false;     // collecting the stream's next rows (the pending slot)
    int nb = 0, W = 0;
    bool windows_api = false;
    std::vector<int64_t> win_start;   // stream sample of each window's first row
    std::vector<int64_t> batch_id;
    std::vector<int64_t> drop_before; // spikes earlier than this are dropped (first batch of a segment)
};

struct Handle {
    lss_params p{};
    OssModel m;
    int dev = 0;
    cudaStream_t st = nullptr;
    cudaStream_t st_copy = nullptr;   // host-to-device copies, overlapped with the previous group's kernels
    int C = 0, T = 0, K = 0, nt = 0, nC = 0, Tf = 0, Cin = 0, NT = 0, W = 0, G = 1, cap = 0, max_iters = 50;
    float th = 8.f;
    int64_t dev_bytes = 0;
    std::string err;
    int64_t launches_last = 0;
    int64_t batches_done = 0, spikes_done = 0;
    bool overflow_pending = false;
    double stage_ms[LSS_N_STAGES] = {};
    int64_t groups_timed = 0;

    // static device state
    float *d_WD = nullptr, *d_Wall3 = nullptr, *d_ctcP = nullptr, *d_pre_wf = nullptr, *d_nm = nullptr;
    float *d_wPCA = nullptr, *d_Ucc = nullptr, *d_xc = nullptr, *d_yc = nullptr, *d_cent = nullptr;
    // tf32 splits of the GEMM's fixed operands (tensor-core path)
    float *d_WD_hi = nullptr, *d_WD_lo = nullptr, *d_Wall3_hi = nullptr, *d_Wall3_lo = nullptr;
    bool tc_whiten = false, tc_project = false;   // GEMMs on the tensor cores
    bool tc_highpass = false;                     // circular high-pass as a tensor-core band GEMM
    bool tf32_data = false;   // gemm_path 2: activations stored once as TF32, two products per GEMM
    bool bf16_proj = false;   // gemm_path 3: projection on BF16 splits (kind::f16, three products)
    bool bf16_pre = false;    // gemm_path 3: high-pass and whitening on BF16 splits as well
    // gemm_path 4 / 5: the projection as one BF16 (lowp 1) or FP8 e4m3 (lowp 2) product of the
    // split operands' hi parts, accepted candidates re-scored exactly in the matching loop
    int lowp = 0;
    bool lowp_ready = false;            // FP8: scales calibrated, folded templates built
    uint8_t* d_W8 = nullptr;            // [T][K*C] e4m3 templates (scales folded)
    float *d_tau = nullptr, *d_sig = nullptr, *d_isig = nullptr;   // [T] template, [K*C] activation scales
    unsigned* d_colmax = nullptr;       // [K*C] calibration scratch
    // PC features straight from the basis convolution and the accepted spikes, without the
    // residual, whenever Bpc holds the convolution to FP32 accuracy (fp32, or an fp32 / BF16 pair:
    // feat_fmt 0 / 1 / 2); the whitened windows and the residual are then written only for the
    // proposal gate and lss_debug_stage (debug_run)
    bool direct_feat = false;
    int feat_fmt = 0;
    float* d_xcorr = nullptr;           // basis cross-correlation [K][K][2 nt - 1]
    float* d_Wall3T = nullptr;          // Wall3 channel-major [T][C][K]
    bool debug_run = false;
    bool need_z() const { return !direct_feat || gate || debug_run || !tc_whiten || !tc_conv; }
    bool tc_conv = false;     // basis convolution as per-component band GEMMs on the tensor cores
    ConvGeometry conv_g;
    float *d_S_hi = nullptr, *d_S_lo = nullptr;   // its band tiles (tf32 or BF16 split)
    // PC-score cluster rule: centroid features [T_final][nC*K], their squared norms, radius^2
    float *d_cpca = nullptr, *d_cpca_nm = nullptr;
    float cl_r2 = 0.f;
    UmmaOperands* um_whiten = nullptr;
    UmmaOperands* um_project = nullptr;
    int* h_gemm_err = nullptr;                    // mapped: device-side wait timeouts
    int* d_gemm_err = nullptr;
    int64_t *d_iCC = nullptr, *d_iU = nullptr;
    int32_t* d_chan = nullptr;
    // stateful high-pass mode (highpass_mode 1): coefficients, the state entering the next group's
    // first row, the stream time that group must start at to continue the chain
    bool iir = false;
    IirCoeffs iirk{};
    float4* d_iir_state = nullptr;   // [C]
    std::vector<float> iir_pow;      // P^0 .. P^kIirChunk of the chunk transition
    float* d_iir_pow = nullptr;
    int64_t iir_expect = INT64_MIN;
    bool iir_reset = true;           // the next streaming group starts a chain
    std::map<int, TapSet> taps;

    // work buffers
    int Wcap = 0, nbcap = 0;
    size_t raw_rows_cap = 0;
    int16_t* d_raw = nullptr;   // [kSlots][raw_rows_cap][Cin]: each slot's rows on the device
    long long* d_colsum = nullptr;   // [nb][C] integer channel sums (zero between launches)
    int* d_ticket = nullptr;         // [nb][ceil(C / 256)] row blocks done (zero between launches)
    float* d_mean = nullptr;         // [nb][C] channel means
    float *d_Xw = nullptr, *d_Y = nullptr, *d_Z = nullptr, *d_Bpc = nullptr, *d_Bt = nullptr;
    float *d_Y_lo = nullptr, *d_Bpc_lo = nullptr;   // tf32 remainders (tensor-core path)
    float *d_Xt_hi = nullptr, *d_Xt_lo = nullptr;   // channel-major wrapped windows (tensor-core high-pass)
    float *d_Zt_hi = nullptr, *d_Zt_lo = nullptr;   // channel-major whitened windows (tensor-core convolution)
    float* d_split = nullptr;   // partial projections of split-K launches [kSplitK][rows][T]
    float4 *d_iir_zs = nullptr, *d_iir_sin = nullptr;   // stateful high-pass: per-chunk states [chunks][C]
    float* d_Bt0 = nullptr;     // low-precision tiers: the initial scores [nb][W][T]
    uint8_t* d_A8 = nullptr;    // FP8 tier: the quantized data operand [nb][W][K*C]
    MatchScratch sc{};
    MatchOut mo{};
    int64_t work_bytes = 0;

    // output slots (in flight groups) and the finished-spike queue
    std::vector<Slot> slots;
    std::deque<int> inflight;   // slot indices in launch order
    // finished spikes waiting for lss_poll: records [ready_head, ready_tail) of ready_buf, which
    // only grows (its entries are rebuilt in place, never zero-filled again)
    std::vector<lss_spike> ready_buf;
    size_t ready_head = 0, ready_tail = 0;
    size_t ready_count() const { return ready_tail - ready_head; }
    lss_spike* ready_append(size_t n) {
        if (ready_head == ready_tail) ready_head = ready_tail = 0;
        if (ready_head > 0 && ready_tail + n > ready_buf.size()) {
            std::memmove(ready_buf.data(), ready_buf.data() + ready_head, ready_count() * sizeof(lss_spike));
            ready_tail -= ready_head;
            ready_head = 0;
        }
        if (ready_tail + n > ready_buf.size()) ready_buf.resize(ready_tail + n);
        lss_spike* p = ready_buf.data() + ready_tail;
        ready_tail += n;
        return p;
    }

    // stream framing
    bool seg_active = false;
    int64_t seg_s0 = 0, next_batch = 0, expected_ct = 0, batch_counter = 0;
    int pend = -1;              // slot whose pinned staging collects the next group's rows
    int64_t pend_rows = 0;      // rows staged there, from the group's first window row on
    int64_t pend_dev = 0;       // of those, rows [0, pend_dev) are in the slot's device rows already
    std::vector<int16_t> last_row;   // the stream's newest row (right pad of a flushed window)
    cudaEvent_t ev_push = nullptr;   // a caller's page-locked rows have reached the device
    std::vector<int64_t> last_kept;     // per final cluster: last kept spike time (duplicate removal)
    std::vector<char> has_kept;
    PropGate* gate = nullptr;           // learned proposal gate (lss_set_proposal), off when null
    // templates are numbered internally by their position along the probe (tmpl_orig[internal] =
    // the oss_input row), so templates that overlap in space have nearby numbers
    std::vector<int32_t> tmpl_orig;
    // pruned matching tier (match_keep > 0): per-sample lists of internal ids and scores; crowded
    // samples list keep_list (> keep) templates when match_keep_wide is set
    int keep = 0, keep_list = 0;
    float crowd_cf = 0.f;
    uint16_t* d_lid = nullptr;          // [nb][W][kPruneKeepMax] internal template ids
    float* d_lsc = nullptr;             // [nb][W][kPruneKeepMax] scores
    float* d_pcf = nullptr;             // [nb][W + 2nt] per-sample maxima of windows too long for shared memory
    unsigned char* d_pslot = nullptr;   // [nb][W]

    ~Handle();
    void init(const char* dir, const lss_params* prm);
    TapSet& taps_for(int Wn);
    void ensure_work(int Wn, int nb);
    // chunks of the stateful high-pass for any group up to nba windows of up to Wa samples
    size_t iir_chunk_cap(int Wa, int nba) const {
        return (size_t)nba * (size_t)((std::max(Wa, NT) + kIirChunk - 1) / kIirChunk) + 1;
    }
    void free_work();
    int acquire_slot();
    void launch_group(Slot& s, int nb, int Wn, int NTs, const TapSet& ts, int stage_rows,
                      const int16_t* dev_src = nullptr, bool rows_on_copy_stream = false);
    void push_device(const int16_t* rows, int64_t n_batches, int64_t first_row_sample);
    void collect(int slot_idx, std::vector<lss_spike>* direct, std::vector<int64_t>* counts);
    void alloc_slot(Slot& s);
    void drain_all();
    void push(const int16_t* x, int64_t n, int64_t ct);
    void flush();
    Slot& pending_slot();
    void launch_pending(int g, int pad_mode);
    int16_t* slot_raw(const Slot& s) { return d_raw + (size_t)(&s - slots.data()) * raw_rows_cap * Cin; }
    void stage_to_device(Slot& s, int64_t upto);
    void run_zero_phase(const int16_t* raw, int nb, int Wn, int NTs, const TapSet& ts, int64_t& nl,
                        const std::function<void()>& mark);
    void run_stages_to_scores(const int16_t* raw, int nb, int Wn, int NTs, const TapSet& ts, int64_t& nl,
                              const std::function<void()>& mark);
    void run_match(int nb, int Wn, int64_t& nl);
};

Handle::~Handle() {
    if (dev >= 0) cudaSetDevice(dev);
    if (st_copy) cudaStreamSynchronize(st_copy);
    if (st) cudaStreamSynchronize(st);
    free_work();
    if (gate) prop_gate_destroy(gate);
    for (auto& kv : taps) {
        cudaFree(kv.second.d);
        for (int v = 0; v < 2; ++v) {
            if (kv.second.g_hi[v]) cudaFree(kv.second.g_hi[v]);
            if (kv.second.g_lo[v]) cudaFree(kv.second.g_lo[v]);
        }
    }
    for (void* p : {(void*)d_xcorr, (void*)d_Wall3T, (void*)d_WD, (void*)d_Wall3, (void*)d_ctcP, (void*)d_pre_wf, (void*)d_nm, (void*)d_wPCA,
                    (void*)d_Ucc, (void*)d_xc, (void*)d_yc, (void*)d_cent, (void*)d_iCC, (void*)d_iU,
                    (void*)d_chan, (void*)d_WD_hi, (void*)d_WD_lo, (void*)d_Wall3_hi, (void*)d_Wall3_lo,
                    (void*)d_S_hi, (void*)d_S_lo, (void*)d_cpca, (void*)d_cpca_nm, (void*)d_iir_state,
                    (void*)d_iir_pow, (void*)d_W8, (void*)d_tau, (void*)d_sig, (void*)d_isig, (void*)d_colmax})
        if (p) cudaFree(p);
    if (h_gemm_err) cudaFreeHost(h_gemm_err);
    for (auto& s : slots) {
        if (s.h_stage) cudaFreeHost(s.h_stage);
        if (s.h_recs) cudaFreeHost(s.h_recs);
        if (s.h_off) cudaFreeHost(s.h_off);
        if (s.h_nsp) cudaFreeHost(s.h_nsp);
        if (s.h_status) cudaFreeHost(s.h_status);
        if (s.ev) cudaEventDestroy(s.ev);
        if (s.ev_copy) cudaEventDestroy(s.ev_copy);
        for (cudaEvent_t e : s.tev)
            if (e) cudaEventDestroy(e);
    }
    if (ev_push) cudaEventDestroy(ev_push);
    if (st_copy) cudaStreamDestroy(st_copy);
    if (st) cudaStreamDestroy(st);
}

void Handle::free_work() {
    umma_free(um_whiten);
    umma_free(um_project);
    um_whiten = um_project = nullptr;
    for (auto& kv : taps) {
        for (int v = 0; v < 2; ++v) {
            umma_free(kv.second.um[v]);
            kv.second.um[v] = nullptr;
        }
        conv_tc_free(kv.second.conv);
        kv.second.conv = nullptr;
    }
    for (void* p : {(void*)d_raw, (void*)d_colsum, (void*)d_ticket, (void*)d_mean, (void*)d_Xw, (void*)d_Y, (void*)d_Z, (void*)d_Bpc, (void*)d_Bt,
                    (void*)d_Y_lo, (void*)d_Bpc_lo, (void*)d_Xt_hi, (void*)d_Xt_lo, (void*)d_Zt_hi, (void*)d_Zt_lo,
                    (void*)d_split, (void*)d_lid, (void*)d_lsc, (void*)d_pcf, (void*)d_pslot, (void*)d_iir_zs,
                    (void*)d_iir_sin, (void*)d_Bt0, (void*)d_A8,
                    (void*)sc.cfmax, (void*)sc.at_t, (void*)sc.at_amp, (void*)mo.n_spikes, (void*)mo.n_iters, (void*)mo.status, (void*)mo.sp_w,
                    (void*)mo.sp_t, (void*)mo.sp_amp, (void*)mo.sp_iter})
        if (p) cudaFree(p);
    d_raw = nullptr;
    d_colsum = nullptr;
    d_ticket = nullptr;
    d_mean = nullptr;
    d_Xw = d_Y = d_Z = d_Bpc = d_Bt = nullptr;
    d_Y_lo = d_Bpc_lo = nullptr;
    d_Xt_hi = d_Xt_lo = nullptr;
    d_Zt_hi = d_Zt_lo = nullptr;
    d_split = nullptr;
    d_iir_zs = d_iir_sin = nullptr;
    d_Bt0 = nullptr;
    d_A8 = nullptr;
    d_lid = nullptr;
    d_lsc = nullptr;
    d_pcf = nullptr;
    d_pslot = nullptr;
    sc = MatchScratch{};
    mo = MatchOut{};
    dev_bytes -= work_bytes;
    work_bytes = 0;
    Wcap = nbcap = 0;
}

// Internal template numbering: by the energy-weighted (y, x) centre of each template on the probe
// (ties by row), so that templates which overlap in space -- the only pairs with a non-negligible
// ctc -- have nearby numbers.  Every template-indexed array of the model is permuted in place;
// orig[internal] = the oss_input row.  Nothing about a template changes, only its number: the
// matching loop's tie rule (the lower number wins an exactly equal Cf) then applies to this
// numbering.
static void renumber_templates(OssModel& m, std::vector<int32_t>& orig) {
    const int64_t T = m.T, K = m.K, C = m.C, nt = m.nt, nC = m.nC, L2 = 2 * m.nt + 1;
    std::vector<double> cy(T), cx(T);
    for (int64_t t = 0; t < T; ++t) {
        double e = 0.0, sy = 0.0, sx = 0.0;
        for (int64_t c = 0; c < C; ++c) {
            double ec = 0.0;
            for (int64_t k = 0; k < K; ++k) {
                const double v = m.Wall3[(t * K + k) * C + c];
                ec += v * v;
            }
            e += ec;
            sy += ec * m.yc[c];
            sx += ec * m.xc[c];
        }
        cy[t] = e > 0.0 ? sy / e : 0.0;
        cx[t] = e > 0.0 ? sx / e : 0.0;
    }
    orig.resize(T);
    for (int64_t t = 0; t < T; ++t) orig[t] = (int32_t)t;
    std::stable_sort(orig.begin(), orig.end(),
                     [&](int32_t a, int32_t b) { return cy[a] < cy[b] || (cy[a] == cy[b] && cx[a] < cx[b]); });
    auto rows = [&](std::vector<float>& a, int64_t len) {
        std::vector<float> o(a.size());
        for (int64_t r = 0; r < T; ++r) std::copy_n(&a[orig[r] * len], len, &o[r * len]);
        a.swap(o);
    };
    rows(m.Wall3, K * C);
    rows(m.pre_wf, nt * C);
    std::vector<float> ctc(m.ctc.size());
    for (int64_t t = 0; t < T; ++t)
        for (int64_t u = 0; u < T; ++u)
            std::copy_n(&m.ctc[((int64_t)orig[t] * T + orig[u]) * L2], L2, &ctc[(t * T + u) * L2]);
    m.ctc.swap(ctc);
    std::vector<int64_t> iU(T);
    for (int64_t t = 0; t < T; ++t) iU[t] = m.iU[orig[t]];
    m.iU.swap(iU);
    std::vector<float> Ucc(m.Ucc.size());
    for (int64_t n = 0; n < nC; ++n)
        for (int64_t t = 0; t < T; ++t)
            std::copy_n(&m.Ucc[(n * T + orig[t]) * K], K, &Ucc[(n * T + t) * K]);
    m.Ucc.swap(Ucc);
}

// The sorter's own limits on a loaded model (beyond the loader's file checks).
static void check_model(const OssModel& m) {
    if (m.nt % 2 == 0) throw LoadError{LSS_ERR_FORMAT, "template length must be odd"};
    if (m.C > 1024) throw LoadError{LSS_ERR_FORMAT, "more than 1024 channels"};
    if (m.K > 8) throw LoadError{LSS_ERR_FORMAT, "more than 8 PCs"};
}

void Handle::init(const char* dir, const lss_params* prm) {
    lss_default_params(&p);
    if (prm) {
        if (prm->abi_version != LSS_ABI_VERSION) throw LoadError{LSS_ERR_ARG, "lss_params.abi_version mismatch"};
        p = *prm;
    }
    if (p.batch_samples <= 0 || p.max_iters <= 0 || p.group_batches <= 0 || p.hp_half_taps < 0)
        throw LoadError{LSS_ERR_ARG, "lss_params: non-positive batch_samples / max_iters / group_batches"};
    m = load_oss_input(dir ? dir : "");
    check_model(m);
    renumber_templates(m, tmpl_orig);
    C = (int)m.C;
    T = (int)m.T;
    K = (int)m.K;
    nt = (int)m.nt;
    nC = (int)m.nC;
    Tf = (int)(m.centroids.size() / 2);
    Cin = p.n_chan_in > 0 ? p.n_chan_in : C;
    if (Cin < C) throw LoadError{LSS_ERR_ARG, "n_chan_in smaller than the channel count"};
    NT = p.batch_samples;
    W = NT + 2 * nt;
    G = p.group_batches;
    max_iters = p.max_iters;
    th = p.th_override > 0.f ? p.th_override : m.th;
    if (p.highpass_mode != 0 && p.highpass_mode != 1)
        throw LoadError{LSS_ERR_ARG, "lss_params.highpass_mode must be 0 (zero-phase) or 1 (stateful sections)"};
    iir = p.highpass_mode == 1;
    if (iir) {
        std::vector<double> sos;
        if (butter_highpass_sos(kHighpassOrder, p.highpass_hz, p.sample_rate_hz, sos) < 0)
            throw LoadError{LSS_ERR_ARG, "lss_params: high-pass edge must lie in (0, sample_rate_hz / 2)"};
        iirk = make_iir_coeffs(sos, iir_pow);
        if (C > 1024) throw LoadError{LSS_ERR_ARG, "the stateful high-pass takes at most 1024 channels"};
    }
    if (Cin > C) {
        for (int64_t v : m.channel_map)
            if (v < 0 || v >= Cin) throw LoadError{LSS_ERR_FORMAT, "channelMap entry outside n_chan_in"};
    }

    dev = p.device;
    int ndev = 0;
    LSS_CUDA(cudaGetDeviceCount(&ndev));
    if (dev < 0 || dev >= ndev) throw LoadError{LSS_ERR_ARG, "device ordinal out of range"};
    LSS_CUDA(cudaSetDevice(dev));
    LSS_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    LSS_CUDA(cudaStreamCreateWithFlags(&st_copy, cudaStreamNonBlocking));

    // derived host arrays: (M @ Wrot) in float64, ctc permuted so the target template is
    // contiguous, squared template norms
    std::vector<float> WD((size_t)C * C);
    for (int i = 0; i < C; ++i)
        for (int j = 0; j < C; ++j) {
            double acc = 0.0;
            for (int k = 0; k < C; ++k) acc += (double)m.drift[(size_t)i * C + k] * (double)m.whitening[(size_t)k * C + j];
            WD[(size_t)i * C + j] = (float)acc;
        }
    const int L2 = 2 * nt + 1;
    std::vector<float> ctcP((size_t)T * L2 * T);
    for (int t = 0; t < T; ++t)
        for (int s = 0; s < T; ++s) {
            const float* src = &m.ctc[((size_t)t * T + s) * L2];
            for (int l = 0; l < L2; ++l) ctcP[((size_t)s * L2 + l) * T + t] = src[l];
        }
    std::vector<float> nm(T);
    for (int t = 0; t < T; ++t) {
        double acc = 0.0;
        for (size_t i = 0; i < (size_t)K * C; ++i) {
            const double v = m.Wall3[(size_t)t * K * C + i];
            acc += v * v;
        }
        nm[t] = (float)acc;
    }
    std::vector<int32_t> chan(C);
    for (int c = 0; c < C; ++c) chan[c] = (int32_t)(Cin > C ? m.channel_map[c] : c);

    d_WD = dev_upload(WD, dev_bytes, st);
    d_Wall3 = dev_upload(m.Wall3, dev_bytes, st);
    d_ctcP = dev_upload(ctcP, dev_bytes, st);
    d_pre_wf = dev_upload(m.pre_wf, dev_bytes, st);
    d_nm = dev_upload(nm, dev_bytes, st);
    d_wPCA = dev_upload(m.wPCA, dev_bytes, st);
    d_Ucc = dev_upload(m.Ucc, dev_bytes, st);
    d_xc = dev_upload(m.xc, dev_bytes, st);
    d_yc = dev_upload(m.yc, dev_bytes, st);
    d_cent = dev_upload(m.centroids, dev_bytes, st);
    d_iCC = dev_upload(m.iCC, dev_bytes, st);
    d_iU = dev_upload(m.iU, dev_bytes, st);
    d_chan = (Cin > C) ? dev_upload(chan, dev_bytes, st) : nullptr;
    // tensor-core GEMMs need K % 16 == 0 and N <= 512 (C for the whitening, T for the projection)
    if (p.gemm_path < 0 || p.gemm_path > 5)
        throw LoadError{LSS_ERR_ARG, "lss_params.gemm_path must be 0 .. 5"};
    if (p.cluster_rule < 0 || p.cluster_rule > 1 || !(p.cluster_radius_um >= 0.f))
        throw LoadError{LSS_ERR_ARG, "lss_params.cluster_rule must be 0 or 1, cluster_radius_um >= 0"};
    if (p.cluster_rule == 1) {
        std::vector<float> cp = load_centroids_pca(dir ? dir : "", m);
        const size_t nf = (size_t)(nC * K);
        std::vector<float> nrm((size_t)Tf);
        for (int j = 0; j < Tf; ++j) {
            double a = 0.0;
            for (size_t q = 0; q < nf; ++q) a += (double)cp[j * nf + q] * cp[j * nf + q];
            nrm[(size_t)j] = (float)a;
        }
        d_cpca = dev_upload(cp, dev_bytes, st);
        d_cpca_nm = dev_upload(nrm, dev_bytes, st);
        const float R = p.cluster_radius_um > 0.f ? p.cluster_radius_um : 80.f;
        cl_r2 = R * R;
    }
    const bool want_tc = p.gemm_path != 1;
    tf32_data = p.gemm_path == 2;
    tc_whiten = want_tc && C % 16 == 0 && C <= 512;
    tc_project = want_tc && (K * C) % 16 == 0 && T <= 512;
    tc_highpass = tc_whiten;
    // the convolution reads the whitened windows the whitening GEMM also writes channel-major;
    // gemm_path 3 runs it and the projection on BF16 splits
    const bool bf16_tier = p.gemm_path >= 3 && (K * C) % 32 == 0;
    lowp = p.gemm_path == 4 ? 1 : (p.gemm_path == 5 ? 2 : 0);
    bf16_pre = bf16_tier && tc_whiten && C % 32 == 0;
    tc_conv = tc_whiten && tc_project && conv_tc_geometry(nt, K, conv_g, bf16_tier);
    if (tc_conv) {
        std::vector<float> S((size_t)conv_g.rows * conv_g.step);
        conv_tc_bands(m.wPCA.data(), K, nt, conv_g, S.data());
        float* d = dev_upload(S, dev_bytes, st);
        d_S_hi = dev_alloc<float>(S.size(), dev_bytes);
        d_S_lo = dev_alloc<float>(S.size(), dev_bytes);
        if (conv_g.bf16)
            launch_split_bf16(d, d_S_hi, d_S_lo, (int64_t)S.size(), st);
        else
            launch_split_tf32(d, d_S_hi, d_S_lo, (int64_t)S.size(), st);
        LSS_CUDA(cudaGetLastError());
        LSS_CUDA(cudaStreamSynchronize(st));
        cudaFree(d);
        dev_bytes -= (int64_t)S.size() * 4;
    }
    // the BF16 projection reads Bpc as the tensor-core convolution writes it (BF16 split)
    bf16_proj = bf16_tier && tc_conv;
    if (tc_whiten || tc_project) {
        if (tc_whiten) {
            d_WD_hi = dev_alloc<float>((size_t)C * C, dev_bytes);
            d_WD_lo = dev_alloc<float>((size_t)C * C, dev_bytes);
            if (bf16_pre)
                launch_split_bf16(d_WD, d_WD_hi, d_WD_lo, (int64_t)C * C, st);
            else
                launch_split_tf32(d_WD, d_WD_hi, d_WD_lo, (int64_t)C * C, st);
        }
        if (tc_project) {
            // two bf16 arrays fit in the halves of the tf32 ones
            d_Wall3_hi = dev_alloc<float>((size_t)T * K * C, dev_bytes);
            d_Wall3_lo = dev_alloc<float>((size_t)T * K * C, dev_bytes);
            if (bf16_proj)
                launch_split_bf16(d_Wall3, d_Wall3_hi, d_Wall3_lo, (int64_t)T * K * C, st);
            else
                launch_split_tf32(d_Wall3, d_Wall3_hi, d_Wall3_lo, (int64_t)T * K * C, st);
        }
        LSS_CUDA(cudaGetLastError());
        LSS_CUDA(cudaStreamSynchronize(st));
    }
    direct_feat = !tf32_data;
    feat_fmt = bf16_proj ? 2 : (tc_project ? 1 : 0);
    if (direct_feat) {
        std::vector<float> P((size_t)K * K * (2 * nt - 1));
        basis_xcorr(m.wPCA.data(), K, nt, P.data());
        d_xcorr = dev_upload(P, dev_bytes, st);
        std::vector<float> UT((size_t)T * C * K);
        for (int t = 0; t < T; ++t)
            for (int k = 0; k < K; ++k)
                for (int c = 0; c < C; ++c) UT[((size_t)t * C + c) * K + k] = m.Wall3[((size_t)t * K + k) * C + c];
        d_Wall3T = dev_upload(UT, dev_bytes, st);
    }
    if (lowp) {
        if (!bf16_proj || (lowp == 2 && (K * C) % 64 != 0))
            throw LoadError{LSS_ERR_ARG, "gemm_path 4 / 5 need the tensor-core convolution and K*C a multiple of 64"};
        if (p.match_keep > 0)
            throw LoadError{LSS_ERR_ARG, "gemm_path 4 / 5 re-score in the full matching loop (match_keep 0)"};
        if (lowp == 2) {
            d_W8 = dev_alloc<uint8_t>((size_t)T * K * C, dev_bytes);
            d_tau = dev_alloc<float>((size_t)T, dev_bytes);
            d_sig = dev_alloc<float>((size_t)K * C, dev_bytes);
            d_isig = dev_alloc<float>((size_t)K * C, dev_bytes);
            d_colmax = dev_alloc<unsigned>((size_t)K * C, dev_bytes);
        }
    }
    if (p.match_keep < 0 || p.match_keep > kPruneKeepMax)
        throw LoadError{LSS_ERR_ARG, "lss_params.match_keep must be 0 (full loop) or 1.." + std::to_string(kPruneKeepMax)};
    keep = std::min(p.match_keep, T);
    if (keep > 0 && T > 1024) throw LoadError{LSS_ERR_ARG, "the pruned matching tier takes at most 1024 templates"};
    if (p.match_keep_wide != 0 && (p.match_keep <= 0 || p.match_keep_wide <= p.match_keep ||
                                   p.match_keep_wide > kPruneKeepMax || !(p.match_keep_crowd >= 0.f)))
        throw LoadError{LSS_ERR_ARG, "lss_params.match_keep_wide must be 0 or in (match_keep, " +
                                         std::to_string(kPruneKeepMax) + "], with match_keep_crowd >= 0"};
    keep_list = keep > 0 && p.match_keep_wide > 0 ? std::min(p.match_keep_wide, T) : keep;
    crowd_cf = p.match_keep_crowd * th * th;
    if (iir) {
        d_iir_state = dev_alloc<float4>((size_t)C, dev_bytes);
        d_iir_pow = dev_upload(iir_pow, dev_bytes, st);
    }
    LSS_CUDA(cudaHostAlloc((void**)&h_gemm_err, sizeof(int), cudaHostAllocMapped | cudaHostAllocPortable));
    *h_gemm_err = 0;
    LSS_CUDA(cudaHostGetDevicePointer((void**)&d_gemm_err, h_gemm_err, 0));
    LSS_CUDA(cudaStreamSynchronize(st));
    m.ctc.clear();
    m.ctc.shrink_to_fit();

    last_kept.assign(Tf, 0);
    has_kept.assign(Tf, 0);
    slots.resize(kSlots);
    for (auto& s : slots) {
        LSS_CUDA(cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming));
        LSS_CUDA(cudaEventCreateWithFlags(&s.ev_copy, cudaEventDisableTiming));
        if (p.profile)
            for (cudaEvent_t& e : s.tev) LSS_CUDA(cudaEventCreate(&e));
    }
    LSS_CUDA(cudaEventCreateWithFlags(&ev_push, cudaEventDisableTiming));
    taps_for(W);
    ensure_work(W, G);
}

TapSet& Handle::taps_for(int Wn) {
    auto it = taps.find(Wn);
    if (it != taps.end()) return it->second;
    std::vector<float> tv;
    int64_t L = 0, R = 0;
    highpass_taps(m.hp_filter, Wn, p.hp_half_taps, tv, L, R);
    tv.resize(((tv.size() + 31) / 32) * 32, 0.f);   // the FIR kernel reads taps in chunks of 32
    TapSet ts;
    ts.L = (int)L;
    ts.R = (int)R;
    ts.d = dev_upload(tv, dev_bytes, st);
    ts.zpitch = (Wn + 7) / 8 * 8;   // 16-byte rows for fp32 and bf16
    if (tc_highpass) {
        const int ntaps = (int)(L + R + 1);
        // rows of 16 bytes; K in whole K-steps (16 fp32 or 32 bf16)
        ts.pitch = (int)(((Wn + L + R) + 7) / 8 * 8);
        const int kstep = bf16_pre ? 32 : 16;
        for (int v = 0; v < 2; ++v) {
            const int TB = kHighpassTile[v];
            const int Kt = ((TB + ntaps - 1) + kstep - 1) / kstep * kstep;
            ts.Kt[v] = Kt;
            std::vector<float> G((size_t)TB * Kt, 0.f);
            for (int j = 0; j < TB; ++j)
                for (int d = 0; d < ntaps; ++d) G[(size_t)j * Kt + j + d] = tv[(size_t)d];
            float* g = dev_upload(G, dev_bytes, st);
            ts.g_hi[v] = dev_alloc<float>(G.size(), dev_bytes);
            ts.g_lo[v] = dev_alloc<float>(G.size(), dev_bytes);
            if (bf16_pre)
                launch_split_bf16(g, ts.g_hi[v], ts.g_lo[v], (int64_t)G.size(), st);
            else
                launch_split_tf32(g, ts.g_hi[v], ts.g_lo[v], (int64_t)G.size(), st);
            LSS_CUDA(cudaGetLastError());
            LSS_CUDA(cudaStreamSynchronize(st));
            cudaFree(g);
            dev_bytes -= (int64_t)G.size() * 4;
        }
    }
    LSS_CUDA(cudaStreamSynchronize(st));
    return taps.emplace(Wn, ts).first->second;
}

void Handle::ensure_work(int Wn, int nb) {
    if (Wn <= Wcap && nb <= nbcap) return;
    if (st) LSS_CUDA(cudaStreamSynchronize(st));
    if (st_copy) LSS_CUDA(cudaStreamSynchronize(st_copy));
    if (pend >= 0 && pend_dev > 0) {
        // the stream's pending rows on the device go back to the slot's staging before the
        // device buffers are replaced
        LSS_CUDA(cudaMemcpy(slots[pend].h_stage, slot_raw(slots[pend]), (size_t)pend_dev * Cin * sizeof(int16_t),
                            cudaMemcpyDeviceToHost));
        pend_dev = 0;
    }
    const int Wa = std::max(Wn, Wcap), nba = std::max(nb, nbcap);
    free_work();
    int64_t before = dev_bytes;
    const int LRmax = Wa;   // wrap rows never exceed the window length
    // one iteration accepts at most one spike per nt + 1 samples (the (2nt+1) max pool), twice
    // that with exact ties
    cap = p.spike_cap > 0 ? p.spike_cap : std::max(2048, 2 * max_iters * ((Wa + nt) / (nt + 1)));
    raw_rows_cap = (size_t)nba * (size_t)std::max(Wa, NT) + 2 * (size_t)nt;
    const int64_t need = (int64_t)kSlots * raw_rows_cap * Cin * 2 + (int64_t)nba * C * 12 + (int64_t)nba * 16 +
                         (int64_t)nba * (Wa + LRmax) * C * 4 + 2LL * nba * Wa * C * 4 +
                         (int64_t)nba * Wa * K * C * 4 * (tc_project && !tf32_data ? 2 : 1) +
                         (int64_t)nba * Wa * C * 4 * (tc_whiten && !tf32_data ? 1 : 0) +
                         (int64_t)nba * ((Wa + 7) / 8 * 8) * C * 4 * (tc_conv ? (tf32_data ? 1 : 2) : 0) +
                         (int64_t)nba * Wa * T * 4 + (int64_t)nba * Wa * 17 + (int64_t)nba * cap * 16 +
                         (tc_project ? (int64_t)kSplitK * std::min(nba, kSplitBatches) * Wa * T * 4 : 0) +
                         (keep > 0 ? (int64_t)nba * Wa * kPruneKeepMax * 6 + (int64_t)nba * (Wa + 2 * nt) * 5 : 0) +
                         (iir ? (int64_t)iir_chunk_cap(Wa, nba) * C * 32 : 0) +
                         (lowp ? (int64_t)nba * Wa * T * 4 + (lowp == 2 ? (int64_t)nba * Wa * K * C : 0) : 0);
    if (p.mem_budget > 0 && dev_bytes + need > p.mem_budget)
        throw LoadError{LSS_ERR_NOMEM, "admission denied: the handle needs " + std::to_string(dev_bytes + need) +
                                           " device bytes, budget " + std::to_string(p.mem_budget)};
    d_raw = dev_alloc<int16_t>((size_t)kSlots * raw_rows_cap * Cin, dev_bytes);
    d_colsum = dev_alloc<long long>((size_t)nba * C, dev_bytes);
    d_ticket = dev_alloc<int>((size_t)nba * ((C + 255) / 256), dev_bytes);
    d_mean = dev_alloc<float>((size_t)nba * C, dev_bytes);
    LSS_CUDA(cudaMemsetAsync(d_colsum, 0, sizeof(long long) * (size_t)nba * C, st));
    LSS_CUDA(cudaMemsetAsync(d_ticket, 0, sizeof(int) * (size_t)nba * ((C + 255) / 256), st));
    if (tc_highpass) {
        // row pitch of any window length up to Wa: W + L + R <= 2W - 1, rounded up to 8
        const size_t n = (size_t)nba * C * (size_t)((2 * Wa + 7) / 8 * 8);
        d_Xt_hi = dev_alloc<float>(n, dev_bytes);
        LSS_CUDA(cudaMemsetAsync(d_Xt_hi, 0, n * sizeof(float), st));
        if (!tf32_data) {
            d_Xt_lo = dev_alloc<float>(n, dev_bytes);
            LSS_CUDA(cudaMemsetAsync(d_Xt_lo, 0, n * sizeof(float), st));
        }
    } else {
        d_Xw = dev_alloc<float>((size_t)nba * (Wa + LRmax) * C, dev_bytes);
    }
    d_Y = dev_alloc<float>((size_t)nba * Wa * C, dev_bytes);
    d_Z = dev_alloc<float>((size_t)nba * Wa * C, dev_bytes);
    if (tc_conv) {
        // any window length up to Wa: rows of W rounded up to 8; the pad columns are never read
        const size_t n = (size_t)nba * C * (size_t)((Wa + 7) / 8 * 8);
        d_Zt_hi = dev_alloc<float>(n, dev_bytes);
        if (!tf32_data) d_Zt_lo = dev_alloc<float>(n, dev_bytes);
    }
    d_Bpc = dev_alloc<float>((size_t)nba * Wa * K * C, dev_bytes);
    d_Bt = dev_alloc<float>((size_t)nba * Wa * T, dev_bytes);
    if (tc_whiten && !tf32_data) d_Y_lo = dev_alloc<float>((size_t)nba * Wa * C, dev_bytes);
    if (tc_project && !tf32_data) d_Bpc_lo = dev_alloc<float>((size_t)nba * Wa * K * C, dev_bytes);
    if (tc_project) d_split = dev_alloc<float>((size_t)kSplitK * std::min(nba, kSplitBatches) * Wa * T, dev_bytes);
    if (iir) {
        const size_t ch = iir_chunk_cap(Wa, nba);
        d_iir_zs = dev_alloc<float4>(ch * C, dev_bytes);
        d_iir_sin = dev_alloc<float4>(ch * C, dev_bytes);
    }
    sc.cfmax = dev_alloc<float>((size_t)nba * Wa, dev_bytes);
    sc.at_t = dev_alloc<int>((size_t)nba * Wa, dev_bytes);
    sc.at_amp = dev_alloc<float>((size_t)nba * Wa, dev_bytes);
    if (keep > 0) {
        d_lid = dev_alloc<uint16_t>((size_t)nba * Wa * kPruneKeepMax, dev_bytes);
        d_lsc = dev_alloc<float>((size_t)nba * Wa * kPruneKeepMax, dev_bytes);
        const int pm = prune_mode(Wa, T, nt, keep_list);
        if (pm < 0) throw LoadError{LSS_ERR_ARG, "window too long for the pruned matching tier"};
        if (!(pm & 1)) {
            d_pcf = dev_alloc<float>((size_t)nba * (Wa + 2 * nt), dev_bytes);
            d_pslot = dev_alloc<unsigned char>((size_t)nba * Wa, dev_bytes);
        }
    }
    mo.n_spikes = dev_alloc<int>(nba, dev_bytes);
    mo.n_iters = dev_alloc<int>(nba, dev_bytes);
    mo.status = dev_alloc<int>(nba, dev_bytes);
    mo.sp_w = dev_alloc<int>((size_t)nba * cap, dev_bytes);
    mo.sp_t = dev_alloc<int>((size_t)nba * cap, dev_bytes);
    mo.sp_amp = dev_alloc<float>((size_t)nba * cap, dev_bytes);
    mo.sp_iter = dev_alloc<int>((size_t)nba * cap, dev_bytes);
    mo.cap = cap;
    if (tc_whiten) {
        um_whiten = bf16_pre ? umma_make_bf16(d_Y, d_Y_lo, (int64_t)nba * Wa, d_WD_hi, d_WD_lo, C, C)
                             : umma_make(d_Y, d_Y_lo, (int64_t)nba * Wa, d_WD_hi, d_WD_lo, C, C);
        if (!um_whiten) throw LoadError{LSS_ERR_INTERNAL, "tensor map setup failed (whitening GEMM)"};
    }
    if (lowp) {
        d_Bt0 = dev_alloc<float>((size_t)nba * Wa * T, dev_bytes);
        if (lowp == 2) d_A8 = dev_alloc<uint8_t>((size_t)nba * Wa * K * C, dev_bytes);
    }
    if (tc_project) {
        um_project = lowp == 2   ? umma_make_lowp(d_A8, (int64_t)nba * Wa, d_W8, T, K * C, 2, d_tau)
                     : lowp == 1 ? umma_make_lowp(d_Bpc, (int64_t)nba * Wa, d_Wall3_hi, T, K * C, 1, nullptr)
                     : bf16_proj
                         ? umma_make_bf16(d_Bpc, d_Bpc_lo, (int64_t)nba * Wa, d_Wall3_hi, d_Wall3_lo, T, K * C)
                         : umma_make(d_Bpc, d_Bpc_lo, (int64_t)nba * Wa, d_Wall3_hi, d_Wall3_lo, T, K * C);
        if (!um_project) throw LoadError{LSS_ERR_INTERNAL, "tensor map setup failed (projection GEMM)"};
    }
    work_bytes = dev_bytes - before;
    Wcap = Wa;
    nbcap = nba;
    // pinned staging + mapped outputs of every idle slot follow the new capacity now, so no
    // later push pays for pinning memory; a slot still in flight is resized when it is reused
    for (auto& s : slots)
        if (!s.busy && !s.reserved) alloc_slot(s);
}

// (re)allocate a slot's pinned staging and host-mapped outputs at the current capacity
void Handle::alloc_slot(Slot& s) {
    if (s.h_stage) cudaFreeHost(s.h_stage), s.h_stage = nullptr;
    if (s.h_recs) cudaFreeHost(s.h_recs), s.h_recs = nullptr;
    if (s.h_off) cudaFreeHost(s.h_off), s.h_off = nullptr;
    if (s.h_nsp) cudaFreeHost(s.h_nsp), s.h_nsp = nullptr;
    if (s.h_status) cudaFreeHost(s.h_status), s.h_status = nullptr;
    s.stage_rows = s.recs_n = 0;
    LSS_CUDA(cudaHostAlloc((void**)&s.h_stage, raw_rows_cap * Cin * sizeof(int16_t), cudaHostAllocPortable));
    LSS_CUDA(cudaHostAlloc((void**)&s.h_recs, (size_t)nbcap * cap * sizeof(SpikeRec),
                           cudaHostAllocMapped | cudaHostAllocPortable));
    LSS_CUDA(cudaHostGetDevicePointer((void**)&s.d_recs, s.h_recs, 0));
    LSS_CUDA(cudaHostAlloc((void**)&s.h_off, (size_t)(nbcap + 1) * sizeof(int),
                           cudaHostAllocMapped | cudaHostAllocPortable));
    LSS_CUDA(cudaHostGetDevicePointer((void**)&s.d_off, s.h_off, 0));
    LSS_CUDA(cudaHostAlloc((void**)&s.h_nsp, (size_t)nbcap * sizeof(int), cudaHostAllocPortable));
    LSS_CUDA(cudaHostAlloc((void**)&s.h_status, (size_t)nbcap * sizeof(int), cudaHostAllocPortable));
    s.stage_rows = raw_rows_cap;
    s.recs_n = (size_t)nbcap * cap;
}

int Handle::acquire_slot() {
    // finish the oldest group if every slot is in flight
    for (;;) {
        for (size_t i = 0; i < slots.size(); ++i)
            if (!slots[i].busy && !slots[i].reserved) {
                Slot& s = slots[i];
                if (!s.h_stage || s.stage_rows < raw_rows_cap || s.recs_n < (size_t)nbcap * cap) alloc_slot(s);
                return (int)i;
            }
        collect(inflight.front(), nullptr, nullptr);
    }
}

// Preprocessing, whitening, basis convolution and projection of nb windows (raw rows already on
// the device) into d_Z (whitened windows) and d_Bt (scores).  mark() is called after each stage.
// Kilosort's preprocessing up to Y (io.py:757-790): channel means, median CAR, circular zero-phase
// high-pass
void Handle::run_zero_phase(const int16_t* raw, int nb, int Wn, int NTs, const TapSet& ts, int64_t& nl,
                            const std::function<void()>& mark) {
    launch_colsum(raw, Cin, d_chan, C, Wn, NTs, nb, d_colsum, d_ticket, d_mean, st), ++nl;
    mark();
    if (tc_highpass) {
        TapSet& tw = const_cast<TapSet&>(ts);
        const int v = nb <= kHighpassSmallGroup ? 0 : 1;
        if (!tw.um[v]) {
            tw.um[v] = bf16_pre ? umma_make_toeplitz_bf16(d_Xt_hi, d_Xt_lo, (int64_t)nbcap * C, tw.pitch,
                                                          kHighpassTile[v], tw.g_hi[v], tw.g_lo[v], tw.Kt[v])
                                : umma_make_toeplitz(d_Xt_hi, d_Xt_lo, (int64_t)nbcap * C, tw.pitch, kHighpassTile[v],
                                                     tw.g_hi[v], tw.g_lo[v], tw.Kt[v]);
            if (!tw.um[v]) throw LoadError{LSS_ERR_INTERNAL, "tensor map setup failed (high-pass band GEMM)"};
        }
        launch_car_t(raw, Cin, d_chan, C, Wn, NTs, nb, d_mean, ts.L, ts.R, tw.pitch, d_Xt_hi, d_Xt_lo, st, bf16_pre),
            ++nl;
        mark();
        LSS_CUDA(launch_umma_highpass(tw.um[v], d_Y, d_Y_lo, nb, C, Wn, d_gemm_err, st));
        ++nl;
        mark();
    } else {
        launch_car(raw, Cin, d_chan, C, Wn, NTs, nb, d_mean, ts.L, ts.R, d_Xw, st), ++nl;
        mark();
        launch_highpass(d_Xw, C, Wn, ts.L, ts.R, ts.d, nb, d_Y, st, tc_whiten ? d_Y_lo : nullptr), ++nl;
        mark();
    }
}

void Handle::run_stages_to_scores(const int16_t* raw, int nb, int Wn, int NTs, const TapSet& ts, int64_t& nl,
                                  const std::function<void()>& mark) {
    if (iir) {
        // stateful high-pass + median CAR straight into Y (timed as the high-pass stage); windows
        // of the windows API (NTs == Wn) are chains of their own, a streaming group continues the
        // previous one unless a segment starts
        IirGroup g{};
        g.nb = nb, g.W = Wn, g.NT = NTs, g.span = (nb - 1) * NTs + Wn;
        g.independent = NTs == Wn;
        g.reset = iir_reset;
        g.carry_row = nb * NTs;
        mark();
        mark();
        const int mode = bf16_pre ? 2 : (tc_whiten ? 1 : 0);
        LSS_CUDA(launch_iir_car(raw, Cin, d_chan, C, g, iirk, d_iir_pow, d_iir_zs, d_iir_sin, d_iir_state, d_Y,
                                tc_whiten ? d_Y_lo : nullptr, mode, st, nl));
        if (!g.independent) iir_reset = false;
        mark();
    } else {
        run_zero_phase(raw, nb, Wn, NTs, ts, nl, mark);
    }
    if (tc_whiten)
        LSS_CUDA(launch_umma_gemm_zt(um_whiten, need_z() ? d_Z : nullptr, nb * Wn, C, C, tc_conv ? d_Zt_hi : nullptr,
                                     tc_conv ? d_Zt_lo : nullptr, Wn, ts.zpitch, d_gemm_err, st,
                                     tc_conv && conv_g.bf16));
    else
        launch_sgemm_nt(d_Y, C, (int64_t)Wn * C, d_WD, C, d_Z, C, (int64_t)Wn * C, Wn, C, C, nb, st);
    ++nl;
    mark();
    if (tc_conv) {
        TapSet& tw = const_cast<TapSet&>(ts);
        if (!tw.conv) {
            tw.conv = conv_tc_make(d_Zt_hi, d_Zt_lo, (int64_t)nbcap * C, Wn, tw.zpitch, d_S_hi, d_S_lo, K, conv_g);
            if (!tw.conv) throw LoadError{LSS_ERR_INTERNAL, "tensor map setup failed (basis convolution)"};
        }
        LSS_CUDA(launch_umma_basis_conv(tw.conv, d_Bpc, d_Bpc_lo, tf32_data, nb, C, Wn, d_gemm_err, st, bf16_proj));
    } else {
        launch_basis_conv_host(d_Z, C, Wn, d_wPCA, m.wPCA.data(), K, nt, nb, d_Bpc, st, d_Bpc_lo,
                               tc_project && tf32_data);
    }
    ++nl;
    mark();
    if (lowp == 2) {
        // FP8 operands: scales from this first group, then the data operand quantized
        const int64_t rows = (int64_t)nb * Wn;
        if (!lowp_ready) {
            launch_lowp_calibrate(d_Bpc, d_Bpc_lo, rows, K * C, d_Wall3, T, d_colmax, d_sig, d_isig, d_W8, d_tau, st);
            nl += 3;
            lowp_ready = true;
        }
        launch_lowp_quantize(d_Bpc, d_Bpc_lo, rows, K * C, d_isig, d_A8, st), ++nl;
    }
    if (tc_project && nb <= kSplitBatches) {
        LSS_CUDA(launch_umma_gemm_splitk(um_project, d_Bt, nb * Wn, T, T, d_split, kSplitK, d_gemm_err, st));
        ++nl;   // and the slice sum
    } else if (tc_project)
        LSS_CUDA(launch_umma_gemm(um_project, d_Bt, nb * Wn, T, T, d_gemm_err, st));
    else
        launch_sgemm_nt(d_Bpc, (int64_t)K * C, (int64_t)Wn * K * C, d_Wall3, (int64_t)K * C, d_Bt, T, (int64_t)Wn * T, Wn,
                        T, K * C, nb, st);
    ++nl;
    // the initial low-precision scores, for the exact re-score of accepted candidates
    if (lowp) LSS_CUDA(cudaMemcpyAsync(d_Bt0, d_Bt, sizeof(float) * (size_t)nb * Wn * T, cudaMemcpyDeviceToDevice, st));
    LSS_CUDA(cudaGetLastError());
    mark();
}

// Enqueue the kernels of one group: windows b = 0..nb-1 start at row b*NTs of the staging copy
// (or of dev_src, rows already on the device, or arriving there through the copy stream when
// rows_on_copy_stream).
void Handle::launch_group(Slot& s, int nb, int Wn, int NTs, const TapSet& ts, int stage_rows, const int16_t* dev_src,
                          bool rows_on_copy_stream) {
    const bool prof = p.profile != 0;
    int stage = 0;
    auto mark = [&]() {
        if (prof) LSS_CUDA(cudaEventRecord(s.tev[stage], st));
        ++stage;
    };
    mark();
    const int16_t* raw = dev_src;
    if (!raw) {
        // the slot's own device rows: the copy runs on the copy stream while the previous group's
        // kernels run (a slot is reused only after its group was collected)
        int16_t* sraw = d_raw + (size_t)(&s - slots.data()) * raw_rows_cap * Cin;
        LSS_CUDA(cudaMemcpyAsync(sraw, s.h_stage, (size_t)stage_rows * Cin * sizeof(int16_t), cudaMemcpyHostToDevice,
                                 st_copy));
        LSS_CUDA(cudaEventRecord(s.ev_copy, st_copy));
        LSS_CUDA(cudaStreamWaitEvent(st, s.ev_copy, 0));
        raw = sraw;
    } else if (rows_on_copy_stream) {
        LSS_CUDA(cudaEventRecord(s.ev_copy, st_copy));
        LSS_CUDA(cudaStreamWaitEvent(st, s.ev_copy, 0));
    }
    mark();
    int64_t nl = 0;
    run_stages_to_scores(raw, nb, Wn, NTs, ts, nl, mark);
    if (gate) nl += prop_gate_run(gate, d_Z, d_Bt, nb, Wn, nt, st);
    run_match(nb, Wn, nl);
    mark();
    launch_rec_offsets(mo, nb, s.d_off, st), ++nl;
    if (direct_feat)
        launch_features_direct(d_Bpc, d_Bpc_lo, feat_fmt, mo, nb, Wn, C, T, K, nt, nC, d_Wall3T, d_xcorr, d_iCC, d_iU,
                               d_Ucc, d_xc, d_yc, d_cent, Tf, d_cpca, d_cpca_nm, cl_r2, s.d_off, s.d_recs, 0, st);
    else
        launch_features(d_Z, mo, nb, Wn, C, T, K, nt, nC, d_wPCA, d_iCC, d_iU, d_Ucc, d_xc, d_yc, d_cent, Tf, d_cpca,
                        d_cpca_nm, cl_r2, s.d_off, s.d_recs, 0, st);
    ++nl;
    LSS_CUDA(cudaGetLastError());
    mark();
    LSS_CUDA(cudaMemcpyAsync(s.h_nsp, mo.n_spikes, sizeof(int) * nb, cudaMemcpyDeviceToHost, st));
    LSS_CUDA(cudaMemcpyAsync(s.h_status, mo.status, sizeof(int) * nb, cudaMemcpyDeviceToHost, st));
    mark();
    LSS_CUDA(cudaEventRecord(s.ev, st));
    s.busy = true;
    s.nb = nb;
    s.W = Wn;
    launches_last += nl;
}

// The matching loop of nb windows on d_Bt (scores): Kilosort's loop over every template, or the
// pruned tier (per-sample lists of the keep best templates, then the loop on them); then d_Z
// becomes the residual, when the features or lss_debug_stage read it.
void Handle::run_match(int nb, int Wn, int64_t& nl) {
    LSS_CUDA(cudaMemsetAsync(mo.status, 0, sizeof(int) * nb, st));
    const bool resid = !direct_feat || debug_run;
    if (keep > 0) {
        launch_prune_select(d_Bt, d_nm, nb, Wn, T, keep, d_lid, d_lsc, st, keep_list, crowd_cf);
        LSS_CUDA(cudaGetLastError());
        LSS_CUDA(launch_match_pruned(d_lid, d_lsc, keep_list, d_ctcP, d_nm, th * th, Wn, T, nt, max_iters, nb, d_pcf,
                                     d_pslot, mo, st));
        nl += 2;   // selection, loop
        if (resid) {
            LSS_CUDA(launch_residual(d_Z, d_pre_wf, mo, Wn, C, nt, nb, st));
            ++nl;
        }
    } else {
        MatchScratch scr = sc;
        if (lowp)
            scr.rs = MatchRescore{d_Bt0, reinterpret_cast<const uint16_t*>(d_Bpc),
                                  reinterpret_cast<const uint16_t*>(d_Bpc_lo), d_Wall3, K * C};
        LSS_CUDA(launch_match(d_Bt, d_Z, d_ctcP, d_pre_wf, d_nm, th * th, Wn, T, C, nt, max_iters, nb, scr, mo, st,
                              p.match_variant, resid));
        nl += resid ? 2 : 1;   // the loop (and the residual)
    }
}

void Handle::push_device(const int16_t* rows, int64_t n_batches, int64_t first_row_sample) {
    if (!rows || n_batches <= 0) throw LoadError{LSS_ERR_ARG, "lss_push_device_span: bad rows / n_batches"};
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, rows) != cudaSuccess || pa.type != cudaMemoryTypeDevice || pa.device != dev) {
        cudaGetLastError();
        throw LoadError{LSS_ERR_ARG, "lss_push_device_span: rows are not device memory of the handle's device"};
    }
    for (int64_t b0 = 0; b0 < n_batches; b0 += G) {
        const int g = (int)std::min<int64_t>(G, n_batches - b0);
        const int si = acquire_slot();
        Slot& s = slots[si];
        s.windows_api = false;
        s.win_start.assign(g, 0);
        s.batch_id.assign(g, 0);
        s.drop_before.assign(g, INT64_MIN);
        for (int b = 0; b < g; ++b) {
            s.win_start[b] = first_row_sample + (b0 + b) * (int64_t)NT;
            s.batch_id[b] = batch_counter + b;
        }
        // the stateful high-pass continues when these rows follow the previous span's
        iir_reset = s.win_start[0] != iir_expect;
        iir_expect = s.win_start[0] + (int64_t)g * NT;
        launch_group(s, g, W, NT, taps_for(W), 0, rows + (size_t)b0 * NT * Cin);
        inflight.push_back(si);
        batch_counter += g;
    }
}

// Turn a finished group into lss_spike records.  direct != nullptr: windows API (results
// returned to the caller, no duplicate removal); otherwise appended to the ready queue.
void Handle::collect(int si, std::vector<lss_spike>* direct, std::vector<int64_t>* counts) {
    Slot& s = slots[si];
    LSS_CUDA(cudaEventSynchronize(s.ev));
    if (!inflight.empty() && inflight.front() == si) inflight.pop_front();
    if (h_gemm_err && *h_gemm_err) {
        const int code = *h_gemm_err;
        *h_gemm_err = 0;
        s.busy = false;
        throw CudaError{"tensor-core GEMM gave up waiting on its pipeline (code " + std::to_string(code) + ")"};
    }
    if (p.profile && s.tev[0]) {
        for (int i = 0; i < LSS_N_STAGES; ++i) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, s.tev[i], s.tev[i + 1]) == cudaSuccess) stage_ms[i] += ms;
        }
        ++groups_timed;
    }
    const int hw = nt / 2;
    const int nf = nC * K;
    for (int b = 0; b < s.nb; ++b) {
        if (s.h_status[b] & 2) {
            s.busy = false;
            throw LoadError{LSS_ERR_ARG, "window too long for the matching kernel's slice bookkeeping"};
        }
    }
    // per batch: order by (time, template), ties in record order, on small keys; every output
    // record is then built once, in its final place
    struct Key {
        int64_t time;
        int32_t tmpl, i;
        bool operator<(const Key& o) const {
            return time != o.time ? time < o.time : (tmpl != o.tmpl ? tmpl < o.tmpl : i < o.i);
        }
    };
    std::vector<Key> keys;
    for (int b = 0; b < s.nb; ++b) {
        const int n = s.h_off[b + 1] - s.h_off[b];
        if (s.h_status[b] & 1) overflow_pending = true;
        const SpikeRec* recs = s.h_recs + s.h_off[b];
        keys.clear();
        keys.reserve(n);
        for (int i = 0; i < n; ++i) {
            const int64_t t = s.win_start[b] + recs[i].w - hw + m.nt0min;
            if (t < s.drop_before[b]) continue;
            keys.push_back({t, tmpl_orig[recs[i].t], i});
        }
        std::sort(keys.begin(), keys.end());
        auto make = [&](const Key& k, lss_spike& o) {
            const SpikeRec& r = recs[k.i];
            o.time = k.time;
            o.tmpl = k.tmpl;
            o.cluster = r.cluster;
            o.amp = r.amp;
            o.x = r.x;
            o.y = r.y;
            o.batch = (int32_t)s.batch_id[b];
            o.n_feat = nf;
            o.iter = r.iter;
            std::memcpy(o.pcfeat, r.feat, sizeof(float) * nf);
            std::memset(o.pcfeat + nf, 0, sizeof(float) * (LSS_MAX_PCFEAT - nf));
        };
        if (direct) {
            const size_t at = direct->size();
            direct->resize(at + keys.size());
            for (size_t j = 0; j < keys.size(); ++j) make(keys[j], (*direct)[at + j]);
            if (counts) counts->push_back((int64_t)keys.size());
        } else {
            size_t kept = 0;
            for (const Key& k : keys) {
                const int cl = recs[k.i].cluster;
                if (p.dedup && cl >= 0 && cl < Tf) {
                    // Kilosort postprocessing.py:9-30: keep when t >= last kept + dt
                    if (has_kept[cl] && k.time < last_kept[cl] + m.dup_bins) continue;
                    last_kept[cl] = k.time;
                    has_kept[cl] = 1;
                }
                keys[kept++] = k;
            }
            lss_spike* o = ready_append(kept);
            for (size_t j = 0; j < kept; ++j) make(keys[j], o[j]);
        }
        spikes_done += (int64_t)keys.size();
    }
    batches_done += s.nb;
    s.busy = false;
}

void Handle::drain_all() {
    while (!inflight.empty()) collect(inflight.front(), nullptr, nullptr);
}

// The slot that collects the stream's next rows and launches a group when its windows are
// complete.  Its rows gather in its device rows: a caller's page-locked rows are copied there
// directly; pageable rows (and pads) wait in the slot's pinned staging and follow in one copy.
Slot& Handle::pending_slot() {
    if (pend < 0) {
        pend = acquire_slot();
        slots[pend].reserved = true;
        pend_rows = 0;
        pend_dev = 0;
    }
    return slots[pend];
}

// staged rows [pend_dev, upto) of the pending slot to its device rows (copy stream)
void Handle::stage_to_device(Slot& s, int64_t upto) {
    if (upto <= pend_dev) return;
    LSS_CUDA(cudaMemcpyAsync(slot_raw(s) + (size_t)pend_dev * Cin, s.h_stage + (size_t)pend_dev * Cin,
                             (size_t)(upto - pend_dev) * Cin * sizeof(int16_t), cudaMemcpyHostToDevice, st_copy));
    pend_dev = upto;
}

// Launch g windows from the pending staging (rows [0, g*NT + 2nt) from the first window's first
// row).  Rows past the staged ones (only at a flush, g = 1): pad_mode 1 repeats the last row
// (Kilosort's last batch, io.py:626-629); pad_mode 2 leaves them zero, which is what Kilosort does
// when the first batch is also the last one (its ibatch == 0 branch, io.py:621-625, runs first and
// never fills the right side).  The staged rows after the g*NT launched ones start the next
// pending slot.
void Handle::launch_pending(int g, int pad_mode) {
    const int si = pend;
    Slot& s = slots[si];
    const int64_t rows_need = (int64_t)g * NT + 2 * nt;
    const int64_t have = pend_rows;
    if (have < rows_need) {
        if (pad_mode == 0 || have == 0 || g != 1) throw LoadError{LSS_ERR_INTERNAL, "window underflow"};
        for (int64_t r = have; r < rows_need; ++r) {
            if (pad_mode == 2)
                std::memset(s.h_stage + r * Cin, 0, (size_t)Cin * sizeof(int16_t));
            else
                std::memcpy(s.h_stage + r * Cin, last_row.data(), (size_t)Cin * sizeof(int16_t));
        }
    }
    stage_to_device(s, std::max(have, rows_need));
    s.windows_api = false;
    s.win_start.assign(g, 0);
    s.batch_id.assign(g, 0);
    s.drop_before.assign(g, INT64_MIN);
    for (int b = 0; b < g; ++b) {
        const int64_t j = next_batch + b;
        s.win_start[b] = seg_s0 + j * NT - nt;
        s.batch_id[b] = batch_counter + b;
        if (j == 0) s.drop_before[b] = seg_s0;   // Kilosort drops negative times of batch 0
    }
    s.reserved = false;
    pend = -1;
    pend_rows = 0;
    pend_dev = 0;
    iir_reset = next_batch == 0;   // a segment's first group starts the stateful high-pass afresh
    iir_expect = s.win_start[0] + (int64_t)g * NT;
    launch_group(s, g, W, NT, taps_for(W), (int)rows_need, slot_raw(s), true);
    inflight.push_back(si);
    next_batch += g;
    batch_counter += g;
    const int64_t carry = have - (int64_t)g * NT;   // rows of the following windows staged already
    if (carry > 0) {
        // they start the next pending slot: a device copy on the copy stream (the launched group
        // only reads its rows; the new slot is idle, so it is never the launched one)
        Slot& ns = pending_slot();
        if (&ns == &s) throw LoadError{LSS_ERR_INTERNAL, "pending rows carried into a busy slot"};
        LSS_CUDA(cudaMemcpyAsync(slot_raw(ns), slot_raw(s) + (size_t)g * NT * Cin, (size_t)carry * Cin * sizeof(int16_t),
                                 cudaMemcpyDeviceToDevice, st_copy));
        pend_rows = carry;
        pend_dev = carry;
    }
}

void Handle::push(const int16_t* x, int64_t n, int64_t ct) {
    if (n < 0 || (n > 0 && !x)) throw LoadError{LSS_ERR_ARG, "lss_push_batch: bad samples"};
    if (seg_active && ct >= 0 && ct != expected_ct) flush();   // discontinuity: close the segment
    if (n == 0) return;
    if (!seg_active) {
        seg_active = true;
        seg_s0 = ct >= 0 ? ct : expected_ct;
        next_batch = 0;
        Slot& s = pending_slot();
        for (int r = 0; r < nt; ++r) std::memcpy(s.h_stage + (size_t)r * Cin, x, (size_t)Cin * sizeof(int16_t));
        pend_rows = nt;                                        // left pad = first sample
        expected_ct = seg_s0;
    }
    expected_ct += n;
    last_row.assign(x + (size_t)(n - 1) * Cin, x + (size_t)n * Cin);
    // page-locked rows go straight to the device on the copy stream, and the call returns once
    // they are there; pageable rows are copied into the slot's pinned staging
    cudaPointerAttributes pa{};
    const bool pinned = cudaPointerGetAttributes(&pa, x) == cudaSuccess && pa.type == cudaMemoryTypeHost;
    cudaGetLastError();
    bool sync = false;
    const int64_t need = (int64_t)G * NT + 2 * nt;
    while (n > 0) {
        Slot& s = pending_slot();
        const int64_t take = std::min(n, need - pend_rows);
        const size_t bytes = (size_t)take * Cin * sizeof(int16_t);
        if (pinned) {
            stage_to_device(s, pend_rows);   // staged rows ahead of these (pads, pageable pushes)
            LSS_CUDA(cudaMemcpyAsync(slot_raw(s) + (size_t)pend_rows * Cin, x, bytes, cudaMemcpyHostToDevice, st_copy));
            pend_dev = pend_rows + take;
            sync = true;
        } else {
            par_memcpy(s.h_stage + pend_rows * Cin, x, bytes);
        }
        pend_rows += take;
        x += take * Cin;
        n -= take;
        if (pend_rows == need) launch_pending(G, 0);
    }
    if (sync) {
        LSS_CUDA(cudaEventRecord(ev_push, st_copy));
        LSS_CUDA(cudaEventSynchronize(ev_push));
    }
}

void Handle::flush() {
    if (!seg_active) return;
    // staged rows past the nt context rows at the front are pending new samples.  Complete windows
    // go out in groups; a window that runs past the data is padded and launched on its own.
    for (;;) {
        const int64_t rows = pend_rows;
        if (rows - nt <= 0) break;
        const int64_t complete = rows >= W ? (rows - W) / NT + 1 : 0;
        if (complete > 0) {
            launch_pending((int)std::min<int64_t>(complete, G), 0);
        } else {
            launch_pending(1, next_batch == 0 ? 2 : 1);
        }
    }
    seg_active = false;
    if (pend >= 0) slots[pend].reserved = false;
    pend = -1;
    pend_rows = 0;
    pend_dev = 0;
}

}  // namespace lss

// =========================================================================================
// C ABI
// =========================================================================================
using lss::Handle;

struct lss_handle {
    Handle h;
};

namespace lss {
// message of the last failure of a call that has no handle (lss_open, lss_match_noalloc)
thread_local std::string g_handleless_error;
}

#define LSS_TRY(hptr, ...)                                                                         \
    try {                                                                                          \
        __VA_ARGS__;                                                                               \
        return LSS_OK;                                                                             \
    } catch (const lss::LoadError& e) {                                                            \
        (hptr)->h.err = e.msg;                                                                     \
        return e.status;                                                                           \
    } catch (const lss::CudaError& e) {                                                            \
        (hptr)->h.err = e.msg;                                                                     \
        return LSS_ERR_CUDA;                                                                       \
    } catch (const std::bad_alloc&) {                                                              \
        (hptr)->h.err = "host allocation failed";                                                  \
        return LSS_ERR_NOMEM;                                                                      \
    } catch (const std::exception& e) {                                                            \
        (hptr)->h.err = e.what();                                                                  \
        return LSS_ERR_INTERNAL;                                                                   \
    }

extern "C" {

int lss_default_params(lss_params* p) {
    if (!p) return LSS_ERR_ARG;
    std::memset(p, 0, sizeof(*p));
    p->abi_version = LSS_ABI_VERSION;
    p->device = 0;
    p->batch_samples = 1500;
    p->max_iters = 50;
    p->group_batches = 1;
    p->n_chan_in = 0;
    p->hp_half_taps = 0;
    p->dedup = 1;
    p->th_override = 0.f;
    p->spike_cap = 0;
    p->mem_budget = 0;
    p->profile = 0;
    p->match_variant = 0;
    p->gemm_path = 0;
    p->cluster_rule = 0;
    p->cluster_radius_um = 0.f;
    p->match_keep = 0;
    p->highpass_mode = 0;
    p->highpass_hz = 300.f;
    p->sample_rate_hz = 30000.f;
    p->match_keep_wide = 0;
    p->match_keep_crowd = 0.5f;
    return LSS_OK;
}

int lss_open(const char* oss_dir, const lss_params* p, lss_handle** out) {
    if (!out) return LSS_ERR_ARG;
    *out = nullptr;
    lss_handle* h = nullptr;
    try {
        h = new lss_handle();
        h->h.init(oss_dir, p);
        *out = h;
        return LSS_OK;
    } catch (const lss::LoadError& e) {
        lss::g_handleless_error = e.msg;
        delete h;
        return e.status;
    } catch (const lss::CudaError& e) {
        lss::g_handleless_error = e.msg;
        delete h;
        return LSS_ERR_CUDA;
    } catch (const std::exception& e) {
        lss::g_handleless_error = e.what();
        delete h;
        return LSS_ERR_INTERNAL;
    }
}

int lss_get_info(const lss_handle* hp, lss_info* info) {
    if (!hp || !info) return LSS_ERR_ARG;
    const Handle& h = hp->h;
    info->C = h.C;
    info->T = h.T;
    info->T_final = h.Tf;
    info->K = h.K;
    info->nt = h.nt;
    info->nC = h.nC;
    info->nt0min = (int32_t)h.m.nt0min;
    info->dup_bins = (int32_t)h.m.dup_bins;
    info->th = h.th;
    info->NT = h.NT;
    info->W = h.W;
    info->group_batches = h.G;
    info->device_bytes = h.dev_bytes;
    info->batches_done = h.batches_done;
    info->spikes_done = h.spikes_done;
    return LSS_OK;
}

int lss_validate_oss_input(const char* oss_dir, lss_info* info) {
    try {
        const std::string dir = oss_dir ? oss_dir : "";
        const lss::OssModel m = lss::load_oss_input(dir);
        lss::check_model(m);
        if (info) {
            std::memset(info, 0, sizeof(*info));
            info->C = (int32_t)m.C;
            info->T = (int32_t)m.T;
            info->T_final = (int32_t)(m.centroids.size() / 2);
            info->K = (int32_t)m.K;
            info->nt = (int32_t)m.nt;
            info->nC = (int32_t)m.nC;
            info->nt0min = (int32_t)m.nt0min;
            info->dup_bins = (int32_t)m.dup_bins;
            info->th = m.th;
        }
        lss::g_handleless_error.clear();
        return LSS_OK;
    } catch (const lss::LoadError& e) {
        lss::g_handleless_error = e.msg;
        return e.status;
    } catch (const std::bad_alloc&) {
        lss::g_handleless_error = "host allocation failed";
        return LSS_ERR_NOMEM;
    } catch (const std::exception& e) {
        lss::g_handleless_error = e.what();
        return LSS_ERR_INTERNAL;
    }
}

int lss_push_batch(lss_handle* hp, const int16_t* samples, int64_t n_samples, int64_t stream_sample_ct) {
    if (!hp) return LSS_ERR_ARG;
    LSS_TRY(hp, {
        cudaSetDevice(hp->h.dev);
        hp->h.launches_last = 0;
        hp->h.push(samples, n_samples, stream_sample_ct);
    })
}

int lss_flush(lss_handle* hp) {
    if (!hp) return LSS_ERR_ARG;
    LSS_TRY(hp, {
        cudaSetDevice(hp->h.dev);
        hp->h.launches_last = 0;
        hp->h.flush();
    })
}

int lss_poll(lss_handle* hp, lss_spike* out, int64_t cap, int64_t* n_out) {
    if (!hp || !n_out || cap < 0 || (cap > 0 && !out)) return LSS_ERR_ARG;
    *n_out = 0;
    try {
        Handle& h = hp->h;
        cudaSetDevice(h.dev);
        // everything already finished, plus the oldest group if nothing is ready yet
        while (!h.inflight.empty() && cudaEventQuery(h.slots[h.inflight.front()].ev) == cudaSuccess)
            h.collect(h.inflight.front(), nullptr, nullptr);
        if (h.ready_count() == 0 && !h.inflight.empty()) h.collect(h.inflight.front(), nullptr, nullptr);
        const int64_t n = std::min<int64_t>(cap, (int64_t)h.ready_count());
        if (n > 0) std::memcpy(out, h.ready_buf.data() + h.ready_head, (size_t)n * sizeof(lss_spike));
        h.ready_head += (size_t)n;
        *n_out = n;
        if (h.overflow_pending) {
            h.overflow_pending = false;
            h.err = "a batch found more spikes than its spike buffer holds; raise spike_cap";
            return LSS_ERR_OVERFLOW;
        }
        return LSS_OK;
    } catch (const lss::LoadError& e) {
        hp->h.err = e.msg;
        return e.status;
    } catch (const lss::CudaError& e) {
        hp->h.err = e.msg;
        return LSS_ERR_CUDA;
    }
}

int lss_pending(lss_handle* hp, int64_t* n) {
    if (!hp || !n) return LSS_ERR_ARG;
    LSS_TRY(hp, {
        cudaSetDevice(hp->h.dev);
        hp->h.drain_all();
        *n = (int64_t)hp->h.ready_count();
    })
}

int lss_close(lss_handle* hp) {
    if (!hp) return LSS_ERR_ARG;
    delete hp;
    return LSS_OK;
}

const char* lss_last_error(const lss_handle* hp) {
    if (!hp) return lss::g_handleless_error.c_str();
    return hp->h.err.c_str();
}

int lss_sort_windows(lss_handle* hp, const int16_t* windows, int32_t n_windows, int32_t W, lss_spike* out,
                     int64_t cap, int64_t* counts) {
    if (!hp || !windows || n_windows <= 0 || !counts || cap < 0 || (cap > 0 && !out)) return LSS_ERR_ARG;
    Handle& h = hp->h;
    if (W <= 2 * h.nt + 1) {
        h.err = "window shorter than 2*nt+2 samples";
        return LSS_ERR_ARG;
    }
    LSS_TRY(hp, {
        cudaSetDevice(h.dev);
        h.launches_last = 0;
        h.drain_all();
        const int per = std::max(1, h.G);
        h.ensure_work(W, per);
        std::vector<lss_spike> all;
        std::vector<int64_t> cnt;
        for (int w0 = 0; w0 < n_windows; w0 += per) {
            const int g = std::min(per, n_windows - w0);
            const int si = h.acquire_slot();
            lss::Slot& s = h.slots[si];
            lss::par_memcpy(s.h_stage, windows + (size_t)w0 * W * h.Cin, (size_t)g * W * h.Cin * sizeof(int16_t));
            s.windows_api = true;
            s.win_start.assign(g, 0);
            s.drop_before.assign(g, INT64_MIN);
            s.batch_id.resize(g);
            for (int b = 0; b < g; ++b) s.batch_id[b] = w0 + b;
            h.launch_group(s, g, W, W, h.taps_for(W), g * W);
            h.collect(si, &all, &cnt);
        }
        int64_t written = 0;
        for (int i = 0; i < n_windows; ++i) counts[i] = cnt[i];
        for (const lss_spike& o : all) {
            if (written >= cap) break;
            out[written++] = o;
        }
        if ((int64_t)all.size() > cap) throw lss::LoadError{LSS_ERR_ARG, "output capacity too small"};
        if (h.overflow_pending) {
            h.overflow_pending = false;
            throw lss::LoadError{LSS_ERR_OVERFLOW, "a window found more spikes than its spike buffer holds"};
        }
    })
}

int lss_debug_stage(lss_handle* hp, const int16_t* window, int32_t W, int32_t stage, float* out, int64_t out_len) {
    if (!hp || !window || !out) return LSS_ERR_ARG;
    Handle& h = hp->h;
    if (W <= 2 * h.nt + 1) return LSS_ERR_ARG;
    const int64_t need = (stage == LSS_STAGE_SCORES) ? (int64_t)W * h.T : (int64_t)W * h.C;
    if (out_len < need || stage < 1 || stage > 3) return LSS_ERR_ARG;
    LSS_TRY(hp, {
        cudaSetDevice(h.dev);
        h.drain_all();
        h.ensure_work(W, 1);
        // the whitened window and the residual are written for this call
        struct DebugRun {
            lss::Handle& h;
            explicit DebugRun(lss::Handle& hh) : h(hh) { h.debug_run = true; }
            ~DebugRun() { h.debug_run = false; }
        } debug_run(h);
        const int si = h.acquire_slot();
        lss::Slot& s = h.slots[si];
        std::memcpy(s.h_stage, window, (size_t)W * h.Cin * sizeof(int16_t));
        lss::TapSet& ts = h.taps_for(W);
        cudaStream_t st = h.st;
        int16_t* sraw = h.slot_raw(s);   // not the stream's pending slot (reserved)
        LSS_CUDA(cudaMemcpyAsync(sraw, s.h_stage, (size_t)W * h.Cin * 2, cudaMemcpyHostToDevice, st));
        int64_t nl = 0;
        h.run_stages_to_scores(sraw, 1, W, W, ts, nl, [] {});
        if (stage == LSS_STAGE_PREPROCESSED) {
            LSS_CUDA(cudaMemcpyAsync(out, h.d_Z, sizeof(float) * need, cudaMemcpyDeviceToHost, st));
        } else {
            if (stage == LSS_STAGE_SCORES) {
                // columns back in oss_input order
                std::vector<float> bt((size_t)need);
                LSS_CUDA(cudaMemcpyAsync(bt.data(), h.d_Bt, sizeof(float) * need, cudaMemcpyDeviceToHost, st));
                LSS_CUDA(cudaStreamSynchronize(st));
                for (int64_t w = 0; w < W; ++w)
                    for (int t = 0; t < h.T; ++t) out[w * h.T + h.tmpl_orig[t]] = bt[(size_t)w * h.T + t];
            } else {
                h.run_match(1, W, nl);
                LSS_CUDA(cudaMemcpyAsync(out, h.d_Z, sizeof(float) * need, cudaMemcpyDeviceToHost, st));
            }
        }
        LSS_CUDA(cudaGetLastError());
        LSS_CUDA(cudaStreamSynchronize(st));
        if (*h.h_gemm_err) {
            *h.h_gemm_err = 0;
            throw lss::CudaError{"tensor-core GEMM gave up waiting on its pipeline"};
        }
    })
}

int lss_push_device_span(lss_handle* hp, const int16_t* dev_rows, int64_t n_batches, int64_t first_row_sample) {
    if (!hp) return LSS_ERR_ARG;
    LSS_TRY(hp, {
        cudaSetDevice(hp->h.dev);
        hp->h.launches_last = 0;
        hp->h.push_device(dev_rows, n_batches, first_row_sample);
    })
}

int lss_cuda_stream(const lss_handle* hp, void** stream) {
    if (!hp || !stream) return LSS_ERR_ARG;
    *stream = (void*)hp->h.st;
    return LSS_OK;
}

int lss_stage_times(lss_handle* hp, double* ms, int32_t n, int64_t* n_groups) {
    if (!hp || !ms || n < 0) return LSS_ERR_ARG;
    for (int i = 0; i < n && i < LSS_N_STAGES; ++i) ms[i] = hp->h.stage_ms[i];
    if (n_groups) *n_groups = hp->h.groups_timed;
    return LSS_OK;
}

int lss_butter_highpass_sos(int32_t order, double cutoff_hz, double fs_hz, double* sos, int32_t cap_sections,
                            int32_t* n_sections) {
    if (!sos || !n_sections) return LSS_ERR_ARG;
    std::vector<double> v;
    const int n = lss::butter_highpass_sos(order, cutoff_hz, fs_hz, v);
    if (n < 0 || n > cap_sections) return LSS_ERR_ARG;
    std::copy(v.begin(), v.end(), sos);
    *n_sections = n;
    return LSS_OK;
}

int lss_set_proposal(lss_handle* hp, const float* params, float logit_threshold, int32_t dilate) {
    if (!hp) return LSS_ERR_ARG;
    Handle& h = hp->h;
    LSS_TRY(hp, {
        cudaSetDevice(h.dev);
        h.drain_all();   // groups in flight finish with the gate they were launched with
        LSS_CUDA(cudaStreamSynchronize(h.st));
        if (h.gate) lss::prop_gate_destroy(h.gate);
        h.gate = nullptr;
        if (params)
            h.gate = lss::prop_gate_create(h.dev, params, logit_threshold, dilate, h.m.Wall3.data(), h.T, h.K, h.C);
    })
}

int lss_proposal_stats(lss_handle* hp, int64_t* cells, int64_t* open) {
    if (!hp || !cells || !open) return LSS_ERR_ARG;
    Handle& h = hp->h;
    LSS_TRY(hp, {
        cudaSetDevice(h.dev);
        *cells = *open = 0;
        if (h.gate) lss::prop_gate_stats(h.gate, h.st, cells, open);
    })
}

int lss_kernel_launches(const lss_handle* hp, int64_t* n) {
    if (!hp || !n) return LSS_ERR_ARG;
    *n = hp->h.launches_last;
    return LSS_OK;
}

}  // extern "C"
