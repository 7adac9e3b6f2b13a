// oss_subset.cpp -- cutting an oss_input/ directory down to some of its preclustered templates, so a
// stream's device state and per-batch work shrink (admission of more streams under mem_budget).
//
// The selection works on the same shape model as the loader (oss_input.cpp) and on the footprint
// the matcher itself sees: a template's energy on channel c is sum_k Wall3[t][k][c]^2 (what the
// projection weighs channel c by), its strongest channel the one of largest energy, its total
// energy the sum over channels.  Candidates are narrowed first by a probe-channel range (channelMap
// values): rule 0 keeps a template whose strongest channel is in range, rule 1 one with any
// in-range channel whose RMS reaches overlap_frac of its strongest channel's.  Then at most
// max_templates are kept, the most active first -- spikes per preclustered template in
// spike_detection_templates.npy (labels outside [0, unclu_T) ignored), ties by energy then by
// index -- or by energy alone.  The kept list is returned in ascending order.
//
// The writer cuts every file that carries the preclustered axis (the axis table below: which files
// and which axes are the reference exporter's layout, subset_templates.py:47-56) and copies every
// other file byte for byte, then writes subset_manifest.json with the reference tool's manifest
// keys, so a subset directory loads anywhere a full one does.
#include "oss_input.hpp"
#include "../../include/lss_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

namespace lss {

extern thread_local std::string g_handleless_error;   // sorter.cu

namespace fs = std::filesystem;

namespace {

struct AxisRule {
    const char* file;
    int axes[2];
    int n_axes;
};
// the files of the exporter's layout that carry the preclustered-template axis, and on which axes
constexpr AxisRule kAxisTable[] = {
    {"Wall3.npy", {0, 0}, 1},                             // [unclu_T, K, C]
    {"ctc.npy", {0, 1}, 2},                               // [unclu_T, unclu_T, 2M+1]
    {"ctc_permuted.npy", {0, 1}, 2},                      // the same, other lag order
    {"iU.npy", {0, 0}, 1},                                // [unclu_T]
    {"Ucc.npy", {1, 0}, 1},                               // [nC, unclu_T, K]
    {"preclustered_template_waveforms.npy", {0, 0}, 1},   // [unclu_T, M, C]
};
constexpr const char* kActivityFile = "spike_detection_templates.npy";

LoadError err(int st, const std::string& m) { return LoadError{st, m}; }

std::string join(const std::string& d, const std::string& f) { return (fs::path(d) / f).string(); }

// shapes the selection needs, checked like the loader does
struct Shapes {
    int64_t T = 0, K = 0, C = 0, T_final = 0;
};

std::vector<double> channel_energy(const NpyArray& wall, const Shapes& s) {
    const std::vector<float> w = wall.as_f32("Wall3.npy");
    std::vector<double> e((size_t)(s.T * s.C), 0.0);
    for (int64_t t = 0; t < s.T; ++t)
        for (int64_t k = 0; k < s.K; ++k)
            for (int64_t c = 0; c < s.C; ++c) {
                const double v = w[(size_t)((t * s.K + k) * s.C + c)];
                e[(size_t)(t * s.C + c)] += v * v;
            }
    return e;
}

struct Plan {
    std::vector<int32_t> keep;
    std::string ranked;           // "spike count" | "template energy" | "all" | "channel range"
    bool chan = false;
    int32_t lo = 0, hi = 0, rule = 0, in_range = 0, on_channels = 0;
    Shapes sh;
};

Plan make_plan(const std::string& dir, const lss_subset_spec& sp) {
    Plan pl;
    const NpyArray wall = npy_load(join(dir, "Wall3.npy"));
    const NpyArray tmpl = npy_load(join(dir, "templates.npy"));
    if (wall.shape.size() != 3 || tmpl.shape.size() != 3)
        throw err(LSS_ERR_FORMAT, "Wall3.npy / templates.npy: expected 3-D arrays");
    Shapes& s = pl.sh;
    s.T = (int64_t)wall.shape[0], s.K = (int64_t)wall.shape[1], s.C = (int64_t)wall.shape[2];
    s.T_final = (int64_t)tmpl.shape[0];
    if ((int64_t)tmpl.shape[2] != s.C) throw err(LSS_ERR_FORMAT, "templates.npy and Wall3.npy disagree on channels");
    if (sp.max_templates < 0 || (sp.rank != 0 && sp.rank != 1) || (sp.chan_rule != 0 && sp.chan_rule != 1) ||
        !(sp.overlap_frac >= 0.f && sp.overlap_frac <= 1.f))
        throw err(LSS_ERR_ARG, "lss_subset_spec: bad max_templates / rank / chan_rule / overlap_frac");
    const std::vector<double> e = channel_energy(wall, s);
    std::vector<double> total((size_t)s.T, 0.0);
    std::vector<int64_t> strongest((size_t)s.T, 0);
    for (int64_t t = 0; t < s.T; ++t) {
        const double* r = &e[(size_t)(t * s.C)];
        total[(size_t)t] = std::accumulate(r, r + s.C, 0.0);
        strongest[(size_t)t] = std::max_element(r, r + s.C) - r;   // first of equal maxima
    }
    std::vector<int32_t> cand;
    if (sp.chan_lo <= sp.chan_hi) {
        pl.chan = true, pl.lo = sp.chan_lo, pl.hi = sp.chan_hi, pl.rule = sp.chan_rule;
        const NpyArray cm = fs::exists(join(dir, "channelMap.npy")) ? npy_load(join(dir, "channelMap.npy"))
                                                                     : npy_load(join(dir, "channel_map.npy"));
        const std::vector<int64_t> probe = cm.as_i64("channelMap.npy");
        if ((int64_t)probe.size() != s.C) throw err(LSS_ERR_FORMAT, "channelMap.npy: one entry per channel expected");
        std::vector<char> in((size_t)s.C, 0);
        for (int64_t c = 0; c < s.C; ++c) in[(size_t)c] = probe[(size_t)c] >= sp.chan_lo && probe[(size_t)c] <= sp.chan_hi;
        pl.in_range = (int32_t)std::count(in.begin(), in.end(), 1);
        if (pl.in_range == 0)
            throw err(LSS_ERR_ARG, "no probe channel in [" + std::to_string(sp.chan_lo) + ", " +
                                       std::to_string(sp.chan_hi) + "]");
        const double f2 = (double)sp.overlap_frac * (double)sp.overlap_frac;   // RMS ratio -> energy ratio
        for (int64_t t = 0; t < s.T; ++t) {
            const double* r = &e[(size_t)(t * s.C)];
            bool take = in[(size_t)strongest[(size_t)t]];
            if (!take && sp.chan_rule == 1) {
                const double top = r[strongest[(size_t)t]];
                for (int64_t c = 0; c < s.C && !take; ++c) take = in[(size_t)c] && r[c] >= f2 * top && top > 0.0;
            }
            if (take) cand.push_back((int32_t)t);
        }
        pl.on_channels = (int32_t)cand.size();
        if (cand.empty()) throw err(LSS_ERR_ARG, "no preclustered template has support on the channel range");
    } else {
        cand.resize((size_t)s.T);
        std::iota(cand.begin(), cand.end(), 0);
    }
    if (sp.max_templates == 0 || (size_t)sp.max_templates >= cand.size()) {
        pl.keep = cand;
        pl.ranked = (int64_t)cand.size() == s.T ? "all" : "channel range";
        return pl;
    }
    std::vector<int64_t> count((size_t)s.T, 0);
    bool by_activity = sp.rank == 0 && fs::exists(join(dir, kActivityFile));
    if (by_activity) {
        for (int64_t v : npy_load(join(dir, kActivityFile)).as_i64(kActivityFile))
            if (v >= 0 && v < s.T) ++count[(size_t)v];
    }
    std::stable_sort(cand.begin(), cand.end(), [&](int32_t a, int32_t b) {
        if (by_activity && count[(size_t)a] != count[(size_t)b]) return count[(size_t)a] > count[(size_t)b];
        if (total[(size_t)a] != total[(size_t)b]) return total[(size_t)a] > total[(size_t)b];
        return a < b;
    });
    cand.resize((size_t)sp.max_templates);
    std::sort(cand.begin(), cand.end());
    pl.keep = cand;
    pl.ranked = by_activity ? "spike count" : "template energy";
    return pl;
}

// "(a,)" / "(a, b)"
std::string tuple_str(const std::vector<size_t>& v) {
    std::string o = "(";
    for (size_t i = 0; i < v.size(); ++i) o += std::to_string(v[i]) + (v.size() == 1 ? "," : (i + 1 < v.size() ? ", " : ""));
    return o + ")";
}

std::string json_str(const std::string& s) {
    std::string o = "\"";
    for (char ch : s) {
        if (ch == '"' || ch == '\\') o += '\\';
        o += ch;
    }
    return o + "\"";
}

// the rows of a C-ordered array kept along `axis` (cnpy semantics: file order is C order)
std::vector<unsigned char> cut_axis(const NpyArray& a, int axis, const std::vector<int32_t>& keep,
                                    std::vector<size_t>& shape) {
    size_t outer = 1, inner = a.word_size;
    for (int i = 0; i < axis; ++i) outer *= shape[(size_t)i];
    for (size_t i = (size_t)axis + 1; i < shape.size(); ++i) inner *= shape[i];
    const size_t n = shape[(size_t)axis];
    std::vector<unsigned char> out(outer * keep.size() * inner);
    for (size_t o = 0; o < outer; ++o)
        for (size_t j = 0; j < keep.size(); ++j)
            std::memcpy(&out[(o * keep.size() + j) * inner], &a.bytes[(o * n + (size_t)keep[j]) * inner], inner);
    shape[(size_t)axis] = keep.size();
    return out;
}

void npy_write(const std::string& path, char kind, size_t word, const std::vector<size_t>& shape,
               const std::vector<unsigned char>& data) {
    const std::string sh = tuple_str(shape);
    std::string dict = "{'descr': '<" + std::string(1, kind) + std::to_string(word) +
                       "', 'fortran_order': False, 'shape': " + sh + ", }";
    // magic (6) + version (2) + header length (2) + dict + spaces + '\n', a multiple of 64 bytes
    size_t total = 10 + dict.size() + 1;
    const size_t pad = (64 - total % 64) % 64;
    dict.append(pad, ' ');
    dict.push_back('\n');
    std::ofstream f(path, std::ios::binary);
    if (!f) throw err(LSS_ERR_IO, "cannot write " + path);
    const unsigned char head[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    f.write(reinterpret_cast<const char*>(head), 8);
    const uint16_t hl = (uint16_t)dict.size();
    const unsigned char hlb[2] = {(unsigned char)(hl & 0xff), (unsigned char)(hl >> 8)};
    f.write(reinterpret_cast<const char*>(hlb), 2);
    f.write(dict.data(), (std::streamsize)dict.size());
    f.write(reinterpret_cast<const char*>(data.data()), (std::streamsize)data.size());
    if (!f) throw err(LSS_ERR_IO, "short write " + path);
}

}  // namespace
}  // namespace lss

using namespace lss;

void lss_subset_default_spec(lss_subset_spec* s) {
    if (!s) return;
    std::memset(s, 0, sizeof(*s));
    s->chan_lo = 1;
    s->chan_hi = 0;   // empty range: no channel filter
    s->overlap_frac = 0.1f;
}

int lss_subset_plan(const char* oss_dir, const lss_subset_spec* spec, int32_t* keep, int32_t cap, int32_t* n_keep) {
    if (!oss_dir || !spec || !n_keep) return LSS_ERR_ARG;
    try {
        const Plan pl = make_plan(oss_dir, *spec);
        *n_keep = (int32_t)pl.keep.size();
        if (keep && cap < (int32_t)pl.keep.size()) {
            g_handleless_error = "lss_subset_plan: keep has room for " + std::to_string(cap) + " of " +
                                 std::to_string(pl.keep.size());
            return LSS_ERR_OVERFLOW;
        }
        if (keep) std::copy(pl.keep.begin(), pl.keep.end(), keep);
        g_handleless_error.clear();
        return LSS_OK;
    } catch (const LoadError& e) {
        g_handleless_error = e.msg;
        return e.status;
    } catch (const std::exception& e) {
        g_handleless_error = e.what();
        return LSS_ERR_INTERNAL;
    }
}

int lss_subset_write(const char* in_dir, const char* out_dir, const lss_subset_spec* spec) {
    if (!in_dir || !out_dir || !spec) return LSS_ERR_ARG;
    try {
        const Plan pl = make_plan(in_dir, *spec);
        const int64_t T = pl.sh.T;
        if ((int64_t)pl.keep.size() >= T) throw err(LSS_ERR_ARG, "nothing to cut: every preclustered template is kept");
        if (fs::exists(out_dir)) throw err(LSS_ERR_IO, std::string(out_dir) + " exists; not overwritten");
        std::error_code ec;
        fs::create_directories(out_dir, ec);
        if (ec) throw err(LSS_ERR_IO, "cannot create " + std::string(out_dir) + ": " + ec.message());
        std::vector<fs::path> files;
        for (const auto& de : fs::directory_iterator(in_dir))
            if (de.is_regular_file()) files.push_back(de.path());
        std::sort(files.begin(), files.end());
        std::ostringstream actions;
        bool first = true;
        for (const fs::path& src : files) {
            const std::string name = src.filename().string();
            const AxisRule* rule = nullptr;
            for (const AxisRule& r : kAxisTable)
                if (name == r.file) rule = &r;
            std::string act;
            if (rule) {
                NpyArray a = npy_load(src.string());
                if (a.fortran_order) throw err(LSS_ERR_FORMAT, name + ": Fortran-ordered file on a template axis");
                std::vector<size_t> shape = a.shape;
                for (int i = 0; i < rule->n_axes; ++i) {
                    const int ax = rule->axes[i];
                    if ((size_t)ax >= shape.size() || (int64_t)shape[(size_t)ax] != T)
                        throw err(LSS_ERR_FORMAT, name + ": axis " + std::to_string(ax) + " is not unclu_T = " +
                                                      std::to_string(T) + " long");
                    a.bytes = cut_axis(a, ax, pl.keep, shape);
                    a.shape = shape;
                }
                npy_write(join(out_dir, name), a.kind, a.word_size, shape, a.bytes);
                std::vector<size_t> axes(rule->axes, rule->axes + rule->n_axes);
                act = "subset axes " + tuple_str(axes) + " -> " + tuple_str(shape);
            } else {
                fs::copy_file(src, fs::path(out_dir) / name, ec);
                if (ec) throw err(LSS_ERR_IO, "cannot copy " + name + ": " + ec.message());
                act = "copy";
            }
            actions << (first ? "" : ",\n") << "    " << json_str(name) << ": " << json_str(act);
            first = false;
        }
        std::ofstream mf(join(out_dir, "subset_manifest.json"));
        mf << "{\n  \"source\": " << json_str(fs::absolute(in_dir).string()) << ",\n  \"original_unclu_T\": " << T
           << ",\n  \"new_unclu_T\": " << pl.keep.size() << ",\n  \"T_unchanged\": " << pl.sh.T_final
           << ",\n  \"metric\": " << json_str(pl.ranked) << ",\n  \"kept_indices\": [";
        for (size_t i = 0; i < pl.keep.size(); ++i) mf << (i ? ", " : "") << pl.keep[i];
        mf << "],\n  \"actions\": {\n" << actions.str() << "\n  }";
        if (pl.chan)
            mf << ",\n  \"channel_filter\": {\"channel_range\": [" << pl.lo << ", " << pl.hi
               << "], \"channel_criterion\": " << json_str(pl.rule == 0 ? "peak" : "overlap")
               << ", \"probe_channels_in_range\": " << pl.in_range << ", \"templates_on_channels\": " << pl.on_channels
               << "}";
        mf << "\n}\n";
        if (!mf) throw err(LSS_ERR_IO, "cannot write subset_manifest.json");
        g_handleless_error.clear();
        return LSS_OK;
    } catch (const LoadError& e) {
        g_handleless_error = e.msg;
        return e.status;
    } catch (const std::exception& e) {
        g_handleless_error = e.what();
        return LSS_ERR_INTERNAL;
    }
}
