// oss_input.hpp -- loading and validating one Kilosort oss_input/ directory (host side).
//
// The .npy reader keeps cnpy's semantics (External/CNPY/cnpy.cpp:62-73,180-184): shape and
// word size come from the header, the payload is taken in file order as a C-ordered array
// and fortran_order is ignored.  The reference exporter relies on this: drift_matrix.npy is
// saved as get_drift_matrix(...).T (a Fortran-ordered file, run_online_spikes.py:628) and the
// sorter reads its bytes back as M.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace lss {

struct LoadError {
    int status;
    std::string msg;
};

struct NpyArray {
    std::vector<size_t> shape;
    size_t word_size = 0;
    char kind = 0;                // 'f', 'i', 'u', 'b'
    bool fortran_order = false;   // parsed, not applied (cnpy)
    std::vector<unsigned char> bytes;
    size_t count() const;
    std::vector<float> as_f32(const std::string& what) const;     // f4 or f8 -> f32
    std::vector<int64_t> as_i64(const std::string& what) const;   // i4 or i8 -> i64
};

NpyArray npy_load(const std::string& path);   // throws LoadError

// Everything the sorter needs from oss_input/, in host memory.
struct OssModel {
    int64_t C = 0, T = 0, T_final = 0, K = 0, nt = 0, nC = 0;
    int64_t nt0min = 0, dup_bins = 0;
    float th = 0.f;
    std::vector<float> Wall3;       // [T][K][C]
    std::vector<float> ctc;         // [T][T][2nt+1]
    std::vector<float> wPCA;        // [K][nt]
    std::vector<float> pre_wf;      // [T][nt][C]
    std::vector<float> whitening;   // [C][C]
    std::vector<float> drift;       // [C][C]
    std::vector<int64_t> iCC;       // [nC][C]
    std::vector<int64_t> iU;        // [T]
    std::vector<float> Ucc;         // [nC][T][K]
    std::vector<float> hp_filter;   // [L]
    std::vector<float> xc, yc;      // [C]
    std::vector<int64_t> channel_map;   // [C]
    std::vector<float> centroids;   // [T_final][2]
};

// Load and validate every file (shapes cross-checked, word sizes checked like
// SorterHelpers.cpp:24-115); throws LoadError instead of calling exit().
OssModel load_oss_input(const std::string& dir);

// cluster_centroids_pca.npy for the PC-score cluster rule: [T_final][nC * K] float32, each final
// cluster's template PC features on its nearest channels, flattened channel-major
// (OnlineKilosort.py:211-230).  The exporter's per-cluster channel average ([T_final][K],
// run_online_spikes.py:523-573) does not fit the rule's scores and is refused.
std::vector<float> load_centroids_pca(const std::string& dir, const OssModel& m);

// Taps of the circular high-pass for window length W (Kilosort preprocessing.py:138-154
// crop/pad, io.py:771-774 correlation + fftshift): out[j] multiplies x[(w + j - left) mod W];
// left/right are clipped to the cropped kernel's support and to half_taps (half_taps <= 0: the
// shortest half length beyond which every tap is below kTapTail of the centre tap).
constexpr double kTapTail = 1e-8;
void highpass_taps(const std::vector<float>& hp, int64_t W, int64_t half_taps,
                   std::vector<float>& taps, int64_t& left, int64_t& right);

}  // namespace lss
