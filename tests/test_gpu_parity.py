"""Parity of the CUDA path (through the C ABI) with the oracle and with the vendored Kilosort
fixtures.  Tolerances: stage outputs within 2e-5 (preprocessed) / 5e-5 (scores, residual) of
the largest magnitude; spike sets agree at >= 99.5% (same template, |dt| <= 1 sample) with
>= 99.5% of the matched amplitudes within 1e-3 relative of the float64 oracle."""
import numpy as np
import pytest

from livespikesorter_gb300 import sorter, synth
from oracle import ks_oracle as ko

from lss_testutil import agreement, make_dataset, match_spikes, write_oss_from_arrays

pytestmark = pytest.mark.gpu

AGREE = 0.995
ROOT_GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def win(golden_dir):
    return np.load(golden_dir / "ks_window.npz")


@pytest.fixture(scope="module")
def win_oss(win, tmp_path_factory):
    return write_oss_from_arrays(win, tmp_path_factory.mktemp("win") / "oss_input")


@pytest.fixture(scope="module")
def win_sorter(win_oss, win):
    with sorter.OnlineSorter(win_oss, max_iters=int(win["max_iters"]), batch_samples=int(win["NT"])) as s:
        yield s


def _rel_close(got, ref, frac):
    scale = np.abs(ref).max()
    err = np.abs(got - ref).max()
    assert err <= frac * scale, f"max err {err:.3e} vs scale {scale:.3e}"


# ---------------------------------------------------------------- stage parity (golden window)
def test_stage_preprocessed(win_sorter, win):
    oss = ko.oss_from_arrays(win)
    ref = ko.preprocess(win["window"].T, oss)            # float64 oracle
    got = win_sorter.debug_stage(win["window"], sorter.STAGE_PREPROCESSED)
    _rel_close(got.T.astype(np.float64), ref, 2e-5)
    _rel_close(got.T.astype(np.float64), win["X"].astype(np.float64), 2e-5)   # the vendored filter


def test_stage_scores(win_sorter, win):
    oss = ko.oss_from_arrays(win)
    X = ko.preprocess(win["window"].T, oss)
    ref = ko.project(X, win["Wall3"].astype(np.float64), win["wPCA"].astype(np.float64))
    got = win_sorter.debug_stage(win["window"], sorter.STAGE_SCORES)
    _rel_close(got.T.astype(np.float64), ref, 5e-5)


def test_stage_residual(win_sorter, win):
    oss = ko.oss_from_arrays(win)
    r = ko.sort_window(win["window"].T, oss, max_iters=int(win["max_iters"]))
    got = win_sorter.debug_stage(win["window"], sorter.STAGE_RESIDUAL)
    _rel_close(got.T.astype(np.float64), r.match.Xres, 5e-5)


def test_window_spikes_match_kilosort(win_sorter, win):
    """Spikes of the golden window against the vendored run_matching output."""
    nt, nt0 = win["wPCA"].shape[1], int(win["misc"][0])
    (sp,) = win_sorter.sort_windows(win["window"])
    t_ref = win["st"][:, 0] - nt // 2 + nt0
    a, amp_ok, amax = agreement(t_ref, win["st"][:, 1], win["amps"], sp["time"], sp["tmpl"], sp["amp"])
    assert len(sp) == len(win["st"])
    assert a == 1.0 and amp_ok == 1.0, (a, amp_ok, amax)


def test_window_features_and_positions(win_sorter, win):
    oss = ko.oss_from_arrays(win)
    r = ko.sort_window(win["window"].T, oss, max_iters=int(win["max_iters"]))
    (sp,) = win_sorter.sort_windows(win["window"])
    nt, nt0 = oss.wPCA.shape[1], oss.nt0min
    order = np.lexsort((r.match.st[:, 1], r.match.st[:, 0]))
    nf = oss.iCC.shape[0] * oss.wPCA.shape[0]
    tF = r.tF[order].reshape(len(order), -1)
    np.testing.assert_array_equal(sp["time"], r.match.st[order, 0] - nt // 2 + nt0)
    np.testing.assert_allclose(sp["pcfeat"][:, :nf], tF, atol=2e-4 * np.abs(tF).max())
    np.testing.assert_allclose(sp["x"], r.xs[order], atol=5e-3)
    np.testing.assert_allclose(sp["y"], r.ys[order], atol=5e-3)
    clu = ko.nearest_centroid(r.xs[order], r.ys[order], oss.centroids)
    assert (sp["cluster"] == clu).mean() >= 0.99


# ---------------------------------------------------------------- stream (golden Kilosort extract)
def test_stream_matches_kilosort_extract(golden_dir, tmp_path):
    z = np.load(golden_dir / "ks_stream.npz")
    d = write_oss_from_arrays(z, tmp_path / "oss_input")
    with sorter.OnlineSorter(d, batch_samples=int(z["NT"]), max_iters=int(z["max_iters"]), dedup=1) as s:
        sp = s.sort_stream(z["data"], chunk=777)
    keep = z["keep"].astype(bool)
    st = z["st"]
    a, amp_ok, amax = agreement(st[keep, 0], st[keep, 1], st[keep, 2], sp["time"], sp["tmpl"], sp["amp"])
    assert a == 1.0 and amp_ok == 1.0, (a, amp_ok, amax)
    assert np.all(np.diff(sp["time"]) >= 0)


def test_stream_chunking_is_invisible(golden_dir, tmp_path):
    z = np.load(golden_dir / "ks_stream.npz")
    d = write_oss_from_arrays(z, tmp_path / "oss_input")
    outs = []
    for chunk, group in ((0, 1), (333, 1), (1999, 2), (64, 3)):
        with sorter.OnlineSorter(d, batch_samples=int(z["NT"]), max_iters=100, group_batches=group) as s:
            outs.append(s.sort_stream(z["data"], chunk=chunk))
    for o in outs[1:]:
        assert len(o) == len(outs[0])
        for f in ("time", "tmpl", "cluster", "amp", "x", "y", "pcfeat"):
            np.testing.assert_array_equal(o[f], outs[0][f])   # bitwise: deterministic kernels


# ---------------------------------------------------------------- seeded configs vs the oracle
def test_config_small_one_batch(cfg_small):
    d, data, _ = cfg_small
    oss = ko.load_oss_input(d)
    with sorter.OnlineSorter(d, max_iters=50) as s:
        (sp,) = s.sort_windows(data[: 60000 + 122])
    r = ko.sort_window(data[: 60000 + 122].T, oss, max_iters=50)
    nt, nt0 = oss.wPCA.shape[1], oss.nt0min
    a, amp_ok, amax = agreement(r.match.st[:, 0] - nt // 2 + nt0, r.match.st[:, 1], r.match.amps,
                                sp["time"], sp["tmpl"], sp["amp"])
    assert len(r.match.st) > 500
    assert a >= AGREE and amp_ok >= AGREE, (a, amp_ok, amax, len(sp), len(r.match.st))


def test_template_subset_directory(cfg_small, tmp_path):
    """A directory cut to the 40 most active of 64 preclustered templates (lss_subset_write through
    livespikesorter_gb300.subset, in place of the reference's subset_templates.py) sorts like the
    float64 oracle on that same directory."""
    from livespikesorter_gb300 import subset
    d0, data, _ = cfg_small
    d = tmp_path / "sub"
    m = subset.subset_oss_input(d0, d, n=40)
    assert m["new_unclu_T"] == 40
    oss = ko.load_oss_input(d)
    assert oss.Wall3.shape[0] == 40
    with sorter.OnlineSorter(d, max_iters=50) as s:
        (sp,) = s.sort_windows(data[: 60000 + 122])
    r = ko.sort_window(data[: 60000 + 122].T, oss, max_iters=50)
    nt, nt0 = oss.wPCA.shape[1], oss.nt0min
    a, amp_ok, amax = agreement(r.match.st[:, 0] - nt // 2 + nt0, r.match.st[:, 1], r.match.amps,
                                sp["time"], sp["tmpl"], sp["amp"])
    assert len(r.match.st) > 300 and sp["tmpl"].max() < 40
    assert a >= AGREE and amp_ok >= AGREE, (a, amp_ok, amax)


def test_tensor_core_conv_tiles_span_windows(cfg_small):
    """96 channels in a group of five windows: the 128-row (window, channel) tiles of the
    tensor-core basis convolution span two windows each.  The group's spikes agree with each window
    sorted by the float64 oracle -- on the FP32 tensor-core path, the FP32-SIMT path (gemm_path 1)
    and the BF16-split path (3) -- and paths 0 and 1 give the same spikes."""
    d, data, _ = cfg_small
    oss = ko.load_oss_input(d)
    nt, nt0 = oss.wPCA.shape[1], oss.nt0min
    W = 1500 + 2 * nt
    wins = np.stack([data[k * 1500: k * 1500 + W] for k in range(5)])
    outs = {}
    for path in (0, 1, 3):
        with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=5, gemm_path=path) as s:
            outs[path] = s.sort_windows(wins)
    ref, got = [], {0: [], 1: [], 3: []}
    for k in range(5):
        r = ko.sort_window(wins[k].T, oss, max_iters=50)
        off = k * 100_000   # keep the windows apart in one agreement count
        ref.append((r.match.st[:, 0] - nt // 2 + nt0 + off, r.match.st[:, 1], r.match.amps))
        for path in (0, 1, 3):
            sp = outs[path][k]
            got[path].append((sp["time"].astype(np.int64) + off, sp["tmpl"], sp["amp"]))
    cat = lambda parts: [np.concatenate([p[i] for p in parts]) for i in range(3)]
    t_r, k_r, a_r = cat(ref)
    assert len(t_r) > 30
    for path in (0, 1, 3):
        a, amp_ok, amax = agreement(t_r, k_r, a_r, *cat(got[path]))
        assert a >= AGREE and amp_ok >= AGREE, (path, a, amp_ok, amax, len(t_r))
    a, amp_ok, amax = agreement(*cat(got[1]), *cat(got[0]))
    assert a == 1.0 and amp_ok == 1.0, (a, amp_ok, amax)


def test_ragged_shapes_scalar_paths(tmp_path):
    """30 channels and 45 templates -- neither a multiple of 4 nor of 16: the FP32-SIMT GEMMs and
    convolution, the matching loop's map-based subtraction (score rows not float4-aligned) and the
    scalar residual, against the float64 oracle: the stream's spikes and one window's residual."""
    cfg = synth.SynthConfig(n_chan=30, n_units=45, n_samples=3 * 1500 + 300, rate_hz=20.0, whiten_batch=1500,
                            whiten_batches=2, seed=31)
    d, data, _ = make_dataset(cfg, tmp_path)
    oss = ko.load_oss_input(d)
    ref = ko.sort_stream(data, oss, 1500, max_iters=50)
    with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=2) as s:
        sp = s.sort_stream(data)
        xres = s.debug_stage(data[:1622], sorter.STAGE_RESIDUAL)
    k = ref["keep"]
    a, amp_ok, amax = agreement(ref["time"][k], ref["template"][k], ref["amp"][k], sp["time"], sp["tmpl"], sp["amp"])
    assert k.sum() > 40
    assert a >= AGREE and amp_ok >= AGREE, (a, amp_ok, amax, len(sp), int(k.sum()))
    r = ko.sort_window(data[:1622].T, oss, max_iters=50)
    _rel_close(xres.T.astype(np.float64), r.match.Xres, 5e-5)


def test_config_stream_384ch(cfg_stream):
    d, data, _ = cfg_stream
    oss = ko.load_oss_input(d)
    ref = ko.sort_stream(data, oss, 1500, max_iters=50)
    with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=4) as s:
        sp = s.sort_stream(data)
    k = ref["keep"]
    a, amp_ok, amax = agreement(ref["time"][k], ref["template"][k], ref["amp"][k], sp["time"], sp["tmpl"], sp["amp"])
    assert k.sum() > 300
    assert a >= AGREE and amp_ok >= AGREE, (a, amp_ok, amax, len(sp), int(k.sum()))


def test_config_dense_overlapping(cfg_dense):
    d, data, _ = cfg_dense
    oss = ko.load_oss_input(d)
    with sorter.OnlineSorter(d, max_iters=50) as s:
        (sp,) = s.sort_windows(data[: 12000 + 122])
    r = ko.sort_window(data[: 12000 + 122].T, oss, max_iters=50)
    nt, nt0 = oss.wPCA.shape[1], oss.nt0min
    a, amp_ok, amax = agreement(r.match.st[:, 0] - nt // 2 + nt0, r.match.st[:, 1], r.match.amps,
                                sp["time"], sp["tmpl"], sp["amp"])
    assert len(r.match.st) > 800
    assert a >= AGREE and amp_ok >= AGREE, (a, amp_ok, amax, len(sp), len(r.match.st))


def test_config_dense_full_size(tmp_path):
    """The full dense shape -- 384 channels, 1000 templates, one 60000-sample batch, 30 Hz with 30 %
    overlaps (about 60,000 spikes placed).  Against the float64 oracle: its spikes on this seeded
    window are a committed fixture (tests/golden/cfg3_full_oracle.npz, a 4.5-minute CPU run by
    tests/golden/make_cfg3_golden.py), and the FP32 path and the BF16-split tier agree with them at
    >= 99.5 % with amplitudes within 1e-3.  Beside it, size-independent properties: the FP32
    tensor-core path agrees with the FP32-SIMT path and the TF32-data tier, and a second run is
    bitwise identical."""
    cfg = synth.SynthConfig(n_chan=384, n_units=1000, n_samples=60000 + 122, rate_hz=30.0, overlap_frac=0.3,
                            whiten_batch=6000, whiten_batches=3, seed=23)
    d, data, _ = make_dataset(cfg, tmp_path)
    win = data[: 60000 + 122]
    outs = {}
    for path in (0, 1, 2, 3):
        with sorter.OnlineSorter(d, max_iters=50, gemm_path=path) as s:
            outs[path] = s.sort_windows(win)[0]
            if path == 0:
                again = s.sort_windows(win)[0]
    assert 10000 < len(outs[0]) < 90000, len(outs[0])   # 19,147 found on the seeded data
    for path in (1, 2, 3):
        a, amp_ok, amax = agreement(outs[0]["time"], outs[0]["tmpl"], outs[0]["amp"],
                                    outs[path]["time"], outs[path]["tmpl"], outs[path]["amp"])
        assert a >= AGREE and amp_ok >= AGREE, (path, a, amp_ok, amax)
    for f in ("time", "tmpl", "amp", "pcfeat"):
        np.testing.assert_array_equal(again[f], outs[0][f])
    import hashlib
    z = np.load(ROOT_GOLDEN / "cfg3_full_oracle.npz")
    same_input = hashlib.sha256(np.ascontiguousarray(win).tobytes()).hexdigest() == str(z["data_sha256"])
    for path in (0, 3):
        a, amp_ok, amax = agreement(z["time"], z["template"], z["amp"], outs[path]["time"], outs[path]["tmpl"],
                                    outs[path]["amp"])
        assert a >= AGREE and amp_ok >= AGREE, (path, a, amp_ok, amax, len(z["time"]), same_input)


# ---------------------------------------------------------------- edge cases
def test_silent_window_has_no_spikes(win_sorter, win):
    (sp,) = win_sorter.sort_windows(np.zeros_like(win["window"]))
    assert len(sp) == 0


def test_short_stream_and_empty_push(golden_dir, tmp_path):
    z = np.load(golden_dir / "ks_stream.npz")
    d = write_oss_from_arrays(z, tmp_path / "oss_input")
    oss = ko.oss_from_arrays(z)
    data = z["data"][:1900]                     # shorter than one batch
    with sorter.OnlineSorter(d, batch_samples=2000, max_iters=100) as s:
        s.push(data[:0])
        s.push(data)
        assert len(s.poll()) == 0               # nothing launched before the flush
        s.flush()
        sp = s.poll_all()
    ref = ko.sort_stream(data, oss, 2000, max_iters=100)
    k = ref["keep"]
    a, _, _ = agreement(ref["time"][k], ref["template"][k], ref["amp"][k], sp["time"], sp["tmpl"], sp["amp"])
    assert k.sum() > 0 and a == 1.0


def test_discontinuity_starts_a_new_segment(golden_dir, tmp_path):
    z = np.load(golden_dir / "ks_stream.npz")
    d = write_oss_from_arrays(z, tmp_path / "oss_input")
    oss = ko.oss_from_arrays(z)
    A, B = z["data"][:2500], z["data"][3000:]
    with sorter.OnlineSorter(d, batch_samples=2000, max_iters=100) as s:
        s.push(A, 0)
        s.push(B, 3000)                         # jumps: the first segment is flushed
        s.flush()
        sp = s.poll_all()
    ra = ko.sort_stream(A, oss, 2000, max_iters=100)
    rb = ko.sort_stream(B, oss, 2000, max_iters=100)
    t_ref = np.concatenate([ra["time"][ra["keep"]], rb["time"][rb["keep"]] + 3000])
    k_ref = np.concatenate([ra["template"][ra["keep"]], rb["template"][rb["keep"]]])
    a_ref = np.concatenate([ra["amp"][ra["keep"]], rb["amp"][rb["keep"]]])
    a, _, _ = agreement(t_ref, k_ref, a_ref, sp["time"], sp["tmpl"], sp["amp"])
    assert a == 1.0


def test_spike_buffer_overflow_is_reported(win_oss, win):
    with sorter.OnlineSorter(win_oss, max_iters=100, spike_cap=2) as s:
        with pytest.raises(sorter.SorterError) as e:
            s.sort_windows(win["window"])
        assert e.value.status == 6


def test_channel_subset_via_channel_map(golden_dir, tmp_path):
    """n_chan_in > C: the sorter picks channelMap columns out of wider rows (the DataSocket's
    channel subset, dataSocket.h:17-21)."""
    z = np.load(golden_dir / "ks_window.npz")
    d = write_oss_from_arrays(z, tmp_path / "oss_input")
    C = z["window"].shape[1]
    perm = np.random.default_rng(0).permutation(C + 9)[:C].astype(np.int32)
    np.save(d / "channelMap.npy", perm)
    wide = np.zeros((z["window"].shape[0], C + 9), np.int16)
    wide[:, perm] = z["window"]
    with sorter.OnlineSorter(d, max_iters=100) as s0:
        (ref,) = s0.sort_windows(z["window"])
    with sorter.OnlineSorter(d, max_iters=100, n_chan_in=C + 9) as s1:
        (got,) = s1.sort_windows(wide)
    np.testing.assert_array_equal(got["time"], ref["time"])
    np.testing.assert_array_equal(got["amp"], ref["amp"])


def test_admission_by_memory_budget(win_oss):
    with pytest.raises(sorter.SorterError) as e:
        sorter.OnlineSorter(win_oss, mem_budget=1 << 20)
    assert e.value.status == 5


def test_kernel_launch_count(win_oss, win):
    with sorter.OnlineSorter(win_oss, max_iters=100) as s:
        s.sort_windows(win["window"])
        # colsum, CAR, high-pass, whitening, convolution, projection split over K + its slice sum,
        # matching loop, record offsets, features (from the convolution: no residual pass)
        assert s.kernel_launches() == 10


def test_cpp_dropin_replay(golden_dir, tmp_path):
    """The C++ drop-in class (lss::OnlineSpikesV2 over a DataSocket) driven by the replay program
    writes spikeOutput.txt lines "time,cluster,amplitude,y" equal to the Kilosort fixture."""
    import subprocess
    from livespikesorter_gb300 import build
    z = np.load(golden_dir / "ks_stream.npz")
    d = write_oss_from_arrays(z, tmp_path / "oss_input")
    rec = tmp_path / "rec.i16"
    z["data"].astype(np.int16).tofile(rec)
    out = tmp_path / "out"
    r = subprocess.run([str(build.REPLAY), str(d), str(rec), str(z["data"].shape[1]), str(out), str(int(z["NT"])), "613"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rows = np.loadtxt(out / "spikeOutput.txt", delimiter=",", ndmin=2)
    keep = z["keep"].astype(bool)
    st = z["st"][keep]
    order = np.lexsort((st[:, 1], st[:, 0]))
    st = st[order]
    assert rows.shape[0] == len(st)
    np.testing.assert_array_equal(rows[:, 0].astype(np.int64), st[:, 0].astype(np.int64))
    np.testing.assert_array_equal(rows[:, 1].astype(np.int64), z["clu"][keep][order])
    np.testing.assert_allclose(rows[:, 2], st[:, 2], rtol=1e-4)


def test_tensor_core_and_simt_gemms_agree(win_oss, win):
    """gemm_path 0 (tcgen05, 3xTF32: high-pass band GEMM, whitening, convolution, projection) and 1
    (FP32 SIMT) agree within 1e-5 (preprocessed) / 2e-5 (scores) of the largest magnitude -- inside
    the oracle tolerances -- and give the same spikes; the BF16-split path 3 (32 channels: every
    stage on kind::f16) within 5e-5 / 1e-4, with the same spikes."""
    outs = {}
    for path in (0, 1, 3):
        with sorter.OnlineSorter(win_oss, max_iters=int(win["max_iters"]), gemm_path=path) as s:
            outs[path] = (s.debug_stage(win["window"], sorter.STAGE_PREPROCESSED),
                          s.debug_stage(win["window"], sorter.STAGE_SCORES), s.sort_windows(win["window"])[0])
    _rel_close(outs[0][0].astype(np.float64), outs[1][0].astype(np.float64), 1e-5)
    _rel_close(outs[0][1].astype(np.float64), outs[1][1].astype(np.float64), 2e-5)
    a, amp_ok, amax = agreement(outs[1][2]["time"], outs[1][2]["tmpl"], outs[1][2]["amp"],
                                outs[0][2]["time"], outs[0][2]["tmpl"], outs[0][2]["amp"])
    assert a == 1.0 and amp_ok == 1.0, (a, amp_ok, amax)
    _rel_close(outs[3][0].astype(np.float64), outs[1][0].astype(np.float64), 5e-5)
    _rel_close(outs[3][1].astype(np.float64), outs[1][1].astype(np.float64), 1e-4)
    a, amp_ok, amax = agreement(outs[1][2]["time"], outs[1][2]["tmpl"], outs[1][2]["amp"],
                                outs[3][2]["time"], outs[3][2]["tmpl"], outs[3][2]["amp"])
    assert a == 1.0 and amp_ok == 1.0, (a, amp_ok, amax)


def test_pc_score_cluster_rule(cfg_stream, tmp_path):
    """cluster_rule 1 -- the final cluster with the best PC score 2 tF.mu - |mu|^2 among the
    clusters within 80 um (OnlineKilosort.py:233-284) -- against the oracle's restatement on the
    384-channel stream: the spikes agree as on the default rule and their cluster ids agree for
    >= 99.5 % of the matched spikes; a radius no cluster is within gives -1 throughout; and the
    exporter's channel-averaged [T, K] centroid file is refused."""
    import shutil
    d0, data, oss_in = cfg_stream
    d = tmp_path / "oss_input"
    shutil.copytree(d0, d)
    flat = synth.centroids_pca_flat(oss_in)
    np.save(d / "cluster_centroids_pca.npy", flat)
    oss = ko.load_oss_input(d)
    ref = ko.sort_stream(data, oss, 1500, max_iters=50, centroids_pca=flat, radius=80.0)
    with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=4, cluster_rule=1) as s:
        sp = s.sort_stream(data)
    k = ref["keep"]
    a, amp_ok, amax = agreement(ref["time"][k], ref["template"][k], ref["amp"][k], sp["time"], sp["tmpl"], sp["amp"])
    assert k.sum() > 300 and a >= AGREE and amp_ok >= AGREE, (a, amp_ok, amax)
    ri, gi = match_spikes(ref["time"][k], ref["template"][k], sp["time"], sp["tmpl"], 1)
    same = (ref["cluster"][k][ri] == sp["cluster"][gi]).mean()
    assert same >= AGREE, same
    assert (sp["cluster"] >= 0).mean() > 0.5
    with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, cluster_rule=1, cluster_radius_um=1e-3) as s:
        far = s.sort_stream(data[:4000])
    assert len(far) > 0 and np.all(far["cluster"] == -1)
    np.save(d / "cluster_centroids_pca.npy", oss_in.centroids_pca)
    with pytest.raises(sorter.SorterError) as e:
        sorter.OnlineSorter(d, cluster_rule=1)
    assert e.value.status == 3


def test_match_variants_agree(cfg_stream):
    """The matching-loop variants -- scores in L2 with 8-CTA clusters (1) or 16-CTA clusters of 1024
    threads (3), scores in shared memory (2) -- run the same arithmetic in the same order per sample:
    bitwise-equal spikes for three windows at once and an equal residual."""
    d, data, _ = cfg_stream
    wins = np.stack([data[k * 1500: k * 1500 + 1622] for k in (1, 2, 3)])
    outs = {}
    for v in (1, 2, 3):
        with sorter.OnlineSorter(d, match_variant=v, group_batches=3) as s:
            outs[v] = (s.sort_windows(wins), s.debug_stage(wins[0], sorter.STAGE_RESIDUAL))
    for v in (2, 3):
        for a, b in zip(outs[1][0], outs[v][0]):
            assert len(a) == len(b) > 0
            for f in ("time", "tmpl", "amp", "iter", "x", "y", "pcfeat"):
                np.testing.assert_array_equal(a[f], b[f], err_msg=f"variant {v} {f}")
        np.testing.assert_array_equal(outs[1][1], outs[v][1])


@pytest.mark.parametrize("tier", [2, 3])
def test_faster_tiers_agree_with_fp32(cfg_stream, tier):
    """gemm_path 2 feeds the activations to the tensor cores as TF32 alone (two products; the fixed
    matrices keep their FP32 split); gemm_path 3 runs the projection on BF16 splits (three kind::f16
    products).  On the 384-channel / 500-template stream each tier's spikes agree with the FP32
    tensor-core path and with the float64 oracle at >= 99.5 % with >= 99.5 % of amplitudes within
    1e-3 relative, and its scores stay within 1e-3 (path 2) / 1e-4 (path 3) of the largest
    magnitude."""
    d, data, _ = cfg_stream
    outs, scores = {}, {}
    win = data[1500 - 61: 3000 + 61]
    for path in (0, tier):
        with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=4, gemm_path=path) as s:
            outs[path] = s.sort_stream(data)
            scores[path] = s.debug_stage(win, sorter.STAGE_SCORES)
    a, amp_ok, amax = agreement(outs[0]["time"], outs[0]["tmpl"], outs[0]["amp"],
                                outs[tier]["time"], outs[tier]["tmpl"], outs[tier]["amp"])
    assert len(outs[0]) > 300
    assert a >= AGREE and amp_ok >= AGREE, (a, amp_ok, amax)
    _rel_close(scores[tier].astype(np.float64), scores[0].astype(np.float64), 1e-3 if tier == 2 else 1e-4)
    # and against the float64 oracle directly, at the same bar as the FP32 path
    ref = ko.sort_stream(data, ko.load_oss_input(d), 1500, max_iters=50)
    k = ref["keep"]
    a, amp_ok, amax = agreement(ref["time"][k], ref["template"][k], ref["amp"][k],
                                outs[tier]["time"], outs[tier]["tmpl"], outs[tier]["amp"])
    assert a >= AGREE and amp_ok >= AGREE, (a, amp_ok, amax)


def test_tensor_core_gemm_384ch(cfg_stream):
    """The 384-channel / 500-template shapes (two N tiles, ragged last M tile) through both paths."""
    d, data, _ = cfg_stream
    win = data[1500 - 61: 3000 + 61]
    outs = {}
    for path in (0, 1):
        with sorter.OnlineSorter(d, gemm_path=path) as s:
            outs[path] = (s.debug_stage(win, sorter.STAGE_PREPROCESSED), s.debug_stage(win, sorter.STAGE_SCORES))
    _rel_close(outs[0][0].astype(np.float64), outs[1][0].astype(np.float64), 1e-5)
    _rel_close(outs[0][1].astype(np.float64), outs[1][1].astype(np.float64), 2e-5)

