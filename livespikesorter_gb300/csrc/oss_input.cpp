// oss_input.cpp -- see oss_input.hpp.
#include "oss_input.hpp"
#include "../../include/lss_gb300.h"

#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>

namespace lss {

static LoadError err(int st, const std::string& m) { return LoadError{st, m}; }

size_t NpyArray::count() const {
    size_t n = 1;
    for (size_t s : shape) n *= s;
    return n;
}

std::vector<float> NpyArray::as_f32(const std::string& what) const {
    std::vector<float> out(count());
    if (kind == 'f' && word_size == 4) {
        std::memcpy(out.data(), bytes.data(), out.size() * 4);
    } else if (kind == 'f' && word_size == 8) {
        const double* d = reinterpret_cast<const double*>(bytes.data());
        for (size_t i = 0; i < out.size(); ++i) out[i] = (float)d[i];
    } else {
        throw err(LSS_ERR_FORMAT, what + ": expected float32/float64 data");
    }
    return out;
}

std::vector<int64_t> NpyArray::as_i64(const std::string& what) const {
    std::vector<int64_t> out(count());
    if (kind == 'i' && word_size == 8) {
        std::memcpy(out.data(), bytes.data(), out.size() * 8);
    } else if (kind == 'i' && word_size == 4) {
        const int32_t* d = reinterpret_cast<const int32_t*>(bytes.data());
        for (size_t i = 0; i < out.size(); ++i) out[i] = d[i];
    } else {
        throw err(LSS_ERR_FORMAT, what + ": expected int32/int64 data");
    }
    return out;
}

NpyArray npy_load(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw err(LSS_ERR_IO, "cannot open " + path);
    unsigned char magic[8];
    f.read(reinterpret_cast<char*>(magic), 8);
    if (!f || magic[0] != 0x93 || std::memcmp(magic + 1, "NUMPY", 5) != 0)
        throw err(LSS_ERR_FORMAT, path + ": not a .npy file");
    uint32_t hlen = 0;
    if (magic[6] == 1) {
        unsigned char b[2];
        f.read(reinterpret_cast<char*>(b), 2);
        hlen = b[0] | (b[1] << 8);
    } else {
        unsigned char b[4];
        f.read(reinterpret_cast<char*>(b), 4);
        hlen = b[0] | (b[1] << 8) | (b[2] << 16) | ((uint32_t)b[3] << 24);
    }
    std::string header(hlen, '\0');
    f.read(&header[0], hlen);
    if (!f) throw err(LSS_ERR_FORMAT, path + ": truncated header");
    NpyArray a;
    size_t p = header.find("'descr'");
    if (p == std::string::npos) throw err(LSS_ERR_FORMAT, path + ": no descr");
    const size_t q1 = header.find('\'', p + 7);   // opening quote of the value
    const size_t q2 = (q1 == std::string::npos) ? q1 : header.find('\'', q1 + 1);
    if (q2 == std::string::npos) throw err(LSS_ERR_FORMAT, path + ": bad descr");
    std::string descr = header.substr(q1 + 1, q2 - q1 - 1);
    if (descr.size() < 3) throw err(LSS_ERR_FORMAT, path + ": bad descr " + descr);
    if (descr[0] == '>') throw err(LSS_ERR_FORMAT, path + ": big-endian data not supported");
    a.kind = descr[1];
    a.word_size = (size_t)std::stoul(descr.substr(2));
    p = header.find("'fortran_order'");
    a.fortran_order = (p != std::string::npos) && header.compare(header.find(':', p) + 1,
                                                                  5, " True") == 0;
    size_t l = header.find('('), r = header.find(')');
    if (l == std::string::npos || r == std::string::npos) throw err(LSS_ERR_FORMAT, path + ": no shape");
    std::string s = header.substr(l + 1, r - l - 1);
    std::stringstream ss(s);
    std::string tok;
    while (std::getline(ss, tok, ',')) {
        size_t i = tok.find_first_not_of(" ");
        if (i == std::string::npos) continue;
        a.shape.push_back((size_t)std::stoull(tok.substr(i)));
    }
    a.bytes.resize(a.count() * a.word_size);
    f.read(reinterpret_cast<char*>(a.bytes.data()), (std::streamsize)a.bytes.size());
    if ((size_t)f.gcount() != a.bytes.size()) throw err(LSS_ERR_FORMAT, path + ": truncated data");
    return a;
}

static std::string join(const std::string& dir, const std::string& name) {
    if (dir.empty()) return name;
    char last = dir.back();
    return (last == '/' || last == '\\') ? dir + name : dir + "/" + name;
}

static void expect_shape(const NpyArray& a, const std::vector<size_t>& want, const std::string& what) {
    if (a.shape != want) {
        std::string got = "(", exp = "(";
        for (size_t s : a.shape) got += std::to_string(s) + ",";
        for (size_t s : want) exp += std::to_string(s) + ",";
        throw err(LSS_ERR_FORMAT, what + ": shape " + got + ") expected " + exp + ")");
    }
}

OssModel load_oss_input(const std::string& dir) {
    OssModel m;
    // misc.txt "key:value" lines (run_online_spikes.py:668-672).  Th_learned is read as a
    // float (Kilosort's value); the reference truncates it with stoi (OnlineSpikesV2.cu:485).
    std::ifstream mf(join(dir, "misc.txt"));
    if (!mf) throw err(LSS_ERR_IO, "cannot open " + join(dir, "misc.txt"));
    std::map<std::string, std::string> kv;
    std::string line;
    while (std::getline(mf, line)) {
        size_t p = line.find(':');
        if (p == std::string::npos) continue;
        std::string v = line.substr(p + 1);
        while (!v.empty() && (v.back() == '\r' || v.back() == ' ')) v.pop_back();
        kv[line.substr(0, p)] = v;
    }
    for (const char* k : {"nt0min", "numNearestChans", "Th_learned", "duplicate_spike_bins"})
        if (!kv.count(k)) throw err(LSS_ERR_FORMAT, std::string("misc.txt: missing ") + k);
    try {
        m.nt0min = (int64_t)std::stod(kv["nt0min"]);
        m.nC = (int64_t)std::stod(kv["numNearestChans"]);
        m.th = (float)std::stod(kv["Th_learned"]);
        m.dup_bins = (int64_t)std::stod(kv["duplicate_spike_bins"]);
    } catch (...) {
        throw err(LSS_ERR_FORMAT, "misc.txt: unparsable value");
    }

    auto tmpl = npy_load(join(dir, "templates.npy"));       // [T_final, M, C]
    if (tmpl.shape.size() != 3 || tmpl.kind != 'f' || tmpl.word_size != 4)
        throw err(LSS_ERR_FORMAT, "templates.npy: expected float32 [T, M, C]");
    m.T_final = (int64_t)tmpl.shape[0];
    m.nt = (int64_t)tmpl.shape[1];
    m.C = (int64_t)tmpl.shape[2];
    const size_t C = (size_t)m.C, nt = (size_t)m.nt;

    auto wall = npy_load(join(dir, "Wall3.npy"));
    if (wall.shape.size() != 3) throw err(LSS_ERR_FORMAT, "Wall3.npy: expected [T, K, C]");
    m.T = (int64_t)wall.shape[0];
    m.K = (int64_t)wall.shape[1];
    const size_t T = (size_t)m.T, K = (size_t)m.K, nC = (size_t)m.nC;
    expect_shape(wall, {T, K, C}, "Wall3.npy");
    m.Wall3 = wall.as_f32("Wall3.npy");

    auto ctc = npy_load(join(dir, "ctc.npy"));
    expect_shape(ctc, {T, T, 2 * nt + 1}, "ctc.npy");
    m.ctc = ctc.as_f32("ctc.npy");
    auto wp = npy_load(join(dir, "wPCA.npy"));
    expect_shape(wp, {K, nt}, "wPCA.npy");
    m.wPCA = wp.as_f32("wPCA.npy");
    auto pw = npy_load(join(dir, "preclustered_template_waveforms.npy"));
    expect_shape(pw, {T, nt, C}, "preclustered_template_waveforms.npy");
    m.pre_wf = pw.as_f32("preclustered_template_waveforms.npy");
    auto wm = npy_load(join(dir, "whiteningMat.npy"));
    expect_shape(wm, {C, C}, "whiteningMat.npy");
    m.whitening = wm.as_f32("whiteningMat.npy");
    auto dm = npy_load(join(dir, "drift_matrix.npy"));
    expect_shape(dm, {C, C}, "drift_matrix.npy");
    m.drift = dm.as_f32("drift_matrix.npy");
    auto icc = npy_load(join(dir, "iCC.npy"));
    if (icc.shape.size() != 2 || icc.shape[1] != C || icc.shape[0] < nC)
        throw err(LSS_ERR_FORMAT, "iCC.npy: expected int64 [>=nC, C]");
    {
        auto full = icc.as_i64("iCC.npy");
        m.iCC.assign(full.begin(), full.begin() + (long)(nC * C));   // first nC rows
    }
    auto iu = npy_load(join(dir, "iU.npy"));
    expect_shape(iu, {T}, "iU.npy");
    m.iU = iu.as_i64("iU.npy");
    auto ucc = npy_load(join(dir, "Ucc.npy"));
    if (ucc.shape.size() != 3 || ucc.shape[0] < nC || ucc.shape[1] != T || ucc.shape[2] != K)
        throw err(LSS_ERR_FORMAT, "Ucc.npy: expected float32 [nC, T, K]");
    {
        auto full = ucc.as_f32("Ucc.npy");
        m.Ucc.assign(full.begin(), full.begin() + (long)(nC * T * K));
    }
    auto hp = npy_load(join(dir, "hp_filter.npy"));
    if (hp.shape.size() != 1 || hp.shape[0] < 3) throw err(LSS_ERR_FORMAT, "hp_filter.npy: expected 1-D");
    m.hp_filter = hp.as_f32("hp_filter.npy");
    auto xc = npy_load(join(dir, "xc.npy"));
    expect_shape(xc, {C}, "xc.npy");
    m.xc = xc.as_f32("xc.npy");
    auto yc = npy_load(join(dir, "yc.npy"));
    expect_shape(yc, {C}, "yc.npy");
    m.yc = yc.as_f32("yc.npy");
    auto cm = npy_load(join(dir, "channelMap.npy"));
    if (cm.count() != C || cm.word_size != 4) throw err(LSS_ERR_FORMAT, "channelMap.npy: expected int32 [C]");
    m.channel_map = cm.as_i64("channelMap.npy");
    auto ce = npy_load(join(dir, "cluster_centroids.npy"));
    if (ce.count() % 2 != 0 || ce.count() == 0)
        throw err(LSS_ERR_FORMAT, "cluster_centroids.npy: expected (x, y) pairs");
    m.centroids = ce.as_f32("cluster_centroids.npy");

    if (m.nC < 1 || (size_t)m.nC > C || m.nC * m.K > LSS_MAX_PCFEAT)
        throw err(LSS_ERR_FORMAT, "numNearestChans out of range for the feature record");
    if (!(m.th > 0.f)) throw err(LSS_ERR_FORMAT, "Th_learned must be > 0");
    for (int64_t v : m.iCC)
        if (v < 0 || v >= m.C) throw err(LSS_ERR_FORMAT, "iCC.npy: channel index out of range");
    for (int64_t v : m.iU)
        if (v < 0 || v >= m.C) throw err(LSS_ERR_FORMAT, "iU.npy: channel index out of range");
    return m;
}

std::vector<float> load_centroids_pca(const std::string& dir, const OssModel& m) {
    auto a = npy_load(join(dir, "cluster_centroids_pca.npy"));
    const size_t nf = (size_t)(m.nC * m.K);
    if (a.shape.size() != 2 || a.shape[0] != (size_t)m.T_final || a.shape[1] != nf)
        throw err(LSS_ERR_FORMAT, "cluster_centroids_pca.npy: the PC-score cluster rule needs float32 [T_final, nC*K] "
                                  "(each cluster's template features on its nearest channels, flattened)");
    return a.as_f32("cluster_centroids_pca.npy");
}

void highpass_taps(const std::vector<float>& hp, int64_t W, int64_t half_taps,
                   std::vector<float>& taps, int64_t& left, int64_t& right) {
    // Kernel of length W after crop/pad (preprocessing.py:138-154): hfull[j].  The output is
    // y[i] = sum_j x[(j + i - W//2) mod W] hfull[j]  ->  offset d = j - W//2, tap(d) = hfull[d + W//2]
    // for d in [-W//2, W-1-W//2].
    const int64_t ft = (int64_t)hp.size();
    auto hfull = [&](int64_t j) -> float {
        if (ft < W) {
            int64_t pad = (W - ft) / 2;
            int64_t q = j - pad;
            return (q >= 0 && q < ft) ? hp[(size_t)q] : 0.f;
        } else if (ft > W) {
            int64_t crop = (ft - W) / 2;
            return hp[(size_t)(j + crop)];
        }
        return hp[(size_t)j];
    };
    const int64_t half = W / 2;
    if (half_taps <= 0) {
        // the farthest offset whose tap still reaches kTapTail of the centre tap
        const double c = std::fabs((double)hfull(half));
        half_taps = 1;
        for (int64_t j = 0; j < W; ++j)
            if (std::fabs((double)hfull(j)) >= kTapTail * c) half_taps = std::max<int64_t>(half_taps, std::llabs(j - half));
    }
    left = std::min<int64_t>(half, half_taps);
    right = std::min<int64_t>(W - 1 - half, half_taps);
    taps.resize((size_t)(left + right + 1));
    for (int64_t d = -left; d <= right; ++d) taps[(size_t)(d + left)] = hfull(d + half);
}

}  // namespace lss
