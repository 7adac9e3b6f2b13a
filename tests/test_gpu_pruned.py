"""The pruned matching tier (lss_params.match_keep): Kilosort's matching loop
(template_matching.py:157-198) run, at every sample, on the match_keep templates of largest initial
Cf only.  Its listed scores receive exactly the full loop's updates, so:

* with every template listed (match_keep >= T) its spikes, amplitudes and residual equal the full
  loop's bit for bit, and the vendored Kilosort fixture's spikes;
* with 32 of 500 templates listed (the length the chosen tier runs) its spikes agree with the full
  FP32 loop and with the float64 oracle at >= 99.5 % with >= 99.5 % of amplitudes within 1e-3
  relative (the oracle's own pruned loop puts 32 at 99.9 % and 16 at 99.3 % on 10 Hz windows of
  this shape);
* at 16 and 32 templates its spikes agree with the float64 oracle's pruned loop
  (oracle/precision_oracle.run_matching_variant, same list rule) at >= 99.5 %;
* windows too long for the lists to stay in shared memory (the 60000-sample batch) run the same
  loop on lists in global memory."""
import numpy as np
import pytest

from livespikesorter_gb300 import sorter
from oracle import ks_oracle as ko
from oracle import precision_oracle as po

from lss_testutil import agreement, write_oss_from_arrays

pytestmark = pytest.mark.gpu

AGREE = 0.995


def test_all_templates_listed_equals_full_loop(golden_dir, tmp_path):
    z = np.load(golden_dir / "ks_window.npz")
    d = write_oss_from_arrays(z, tmp_path / "oss_input")
    T = z["Wall3"].shape[0]
    assert T <= 16
    outs = {}
    for keep in (0, 16):   # 16 >= T = 12: every template listed
        with sorter.OnlineSorter(d, max_iters=int(z["max_iters"]), batch_samples=int(z["NT"]), match_keep=keep) as s:
            (sp,) = s.sort_windows(z["window"])
            outs[keep] = (sp, s.debug_stage(z["window"], sorter.STAGE_RESIDUAL))
    a, b = outs[0][0], outs[16][0]
    assert len(a) == len(b) == len(z["st"])
    for f in ("time", "tmpl", "amp", "iter", "x", "y", "pcfeat"):
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)
    np.testing.assert_array_equal(outs[0][1], outs[16][1])
    # and the vendored Kilosort's spikes (the fixture)
    nt, nt0 = z["wPCA"].shape[1], int(z["misc"][0])
    fr, ok, amax = agreement(z["st"][:, 0] - nt // 2 + nt0, z["st"][:, 1], z["amps"], b["time"], b["tmpl"], b["amp"])
    assert fr == 1.0 and ok == 1.0, (fr, ok, amax)


def test_pruned_tier_agrees_with_full_loop_384ch(cfg_stream):
    d, data, _ = cfg_stream
    outs = {}
    for keep in (0, 32):
        with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=4, match_keep=keep) as s:
            outs[keep] = s.sort_stream(data)
    ref, got = outs[0], outs[32]
    assert len(ref) > 300
    a, amp_ok, amax = agreement(ref["time"], ref["tmpl"], ref["amp"], got["time"], got["tmpl"], got["amp"])
    assert a >= AGREE and amp_ok >= AGREE, (a, amp_ok, amax, len(ref), len(got))
    # and the float64 oracle's full loop, at the bar of the FP32 path
    oref = ko.sort_stream(data, ko.load_oss_input(d), 1500, max_iters=50)
    k = oref["keep"]
    a, amp_ok, amax = agreement(oref["time"][k], oref["template"][k], oref["amp"][k], got["time"], got["tmpl"],
                                got["amp"])
    assert a >= AGREE and amp_ok >= AGREE, (a, amp_ok, amax)


@pytest.mark.parametrize("keep", [16, 24, 32])
def test_pruned_tier_against_oracle_pruned_loop(cfg_stream, keep):
    """Window by window against the float64 oracle's pruned loop with the same list rule."""
    d, data, _ = cfg_stream
    oss = ko.load_oss_input(d)
    nt, nt0 = oss.wPCA.shape[1], oss.nt0min
    wins = np.stack([data[k * 1500: k * 1500 + 1622] for k in (1, 2, 3)])
    with sorter.OnlineSorter(d, max_iters=50, group_batches=3, match_keep=keep) as s:
        got = s.sort_windows(wins)
    n_ref = n_match = n_amp = 0.0
    for win, sp in zip(wins, got):
        X = ko.preprocess(win.T, oss)
        st, amps = po.run_matching_variant(X, oss.Wall3, oss.wPCA, oss.ctc, oss.th_learned, keep=keep, max_iters=50)
        a, amp_ok, _ = agreement(st[:, 0] - nt // 2 + nt0, st[:, 1], amps, sp["time"], sp["tmpl"], sp["amp"])
        n_ref += len(st)
        n_match += a * max(len(st), len(sp))
        n_amp += amp_ok * a * max(len(st), len(sp))
    assert n_ref > 300
    assert n_match / n_ref >= AGREE and n_amp / n_match >= AGREE, (n_match / n_ref, n_amp / n_match)


def test_widened_lists(cfg_stream):
    """match_keep_wide: with no sample crowded the spikes are the 16-entry lists' bit for bit (the
    widened loop skips the padding entries); with crowded samples at Th^2 / 2 they agree with the
    float64 oracle's pruned loop under the same rule at >= 99.5 %."""
    d, data, _ = cfg_stream
    oss = ko.load_oss_input(d)
    nt, nt0 = oss.wPCA.shape[1], oss.nt0min
    wins = np.stack([data[k * 1500: k * 1500 + 1622] for k in (1, 2, 3)])
    outs = {}
    for name, kw in (("k16", {}), ("none", dict(match_keep_wide=24, match_keep_crowd=1e30)),
                     ("half", dict(match_keep_wide=24, match_keep_crowd=0.5))):
        with sorter.OnlineSorter(d, max_iters=50, group_batches=3, match_keep=16, **kw) as s:
            outs[name] = s.sort_windows(wins)
    for a, b in zip(outs["k16"], outs["none"]):
        for f in ("time", "tmpl", "amp", "iter", "x", "y", "pcfeat"):
            np.testing.assert_array_equal(a[f], b[f], err_msg=f)
    n_ref = n_match = n_amp = 0.0
    for win, sp in zip(wins, outs["half"]):
        X = ko.preprocess(win.T, oss)
        st, amps = po.run_matching_variant(X, oss.Wall3, oss.wPCA, oss.ctc, oss.th_learned, keep=16, keep_wide=24,
                                           crowd=0.5, max_iters=50)
        a, amp_ok, _ = agreement(st[:, 0] - nt // 2 + nt0, st[:, 1], amps, sp["time"], sp["tmpl"], sp["amp"])
        n_ref += len(st)
        n_match += a * max(len(st), len(sp))
        n_amp += amp_ok * a * max(len(st), len(sp))
    assert n_ref > 300
    assert n_match / n_ref >= AGREE and n_amp / n_match >= AGREE, (n_match / n_ref, n_amp / n_match)


def test_concurrent_pruned_streams_equal_alone(cfg_stream):
    """Eight handles of the chosen tier's arithmetic (BF16 splits, 16 listed templates, 24 at
    crowded samples) pushing single batches from their own host threads at once -- cluster loops of
    different streams sharing SMs, so CTAs of one cluster run at different speeds -- give, bit for
    bit, the spikes one handle gives alone."""
    import threading
    d, data, _ = cfg_stream
    kw = dict(batch_samples=1500, max_iters=50, gemm_path=3, match_keep=16, match_keep_wide=24, match_keep_crowd=0.5)
    with sorter.OnlineSorter(d, **kw) as s:
        alone = s.sort_stream(data, chunk=1500)
    assert len(alone) > 300
    n = 8
    results, errors = [None] * n, []
    barrier = threading.Barrier(n)

    def run(i):
        try:
            with sorter.OnlineSorter(d, **kw) as s:
                barrier.wait()
                got = []
                for pos in range(0, data.shape[0], 1500):
                    s.push(data[pos:pos + 1500])
                    got.append(s.poll())
                s.flush()
                got.append(s.poll_all())
                results[i] = np.concatenate(got)
        except Exception as e:   # surfaced below, after every thread finished
            errors.append(e)

    th = [threading.Thread(target=run, args=(i,)) for i in range(n)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    for got in results:
        assert len(got) == len(alone)
        for f in ("time", "tmpl", "cluster", "amp", "x", "y", "pcfeat"):
            np.testing.assert_array_equal(got[f], alone[f], err_msg=f)


def test_pruned_tier_dense_overlapping(cfg_dense):
    """30 Hz with 30 % of the spikes overlapping: against the float64 oracle's full loop."""
    d, data, _ = cfg_dense
    oss = ko.load_oss_input(d)
    win = data[: 12000 + 122]
    with sorter.OnlineSorter(d, max_iters=50, match_keep=32) as s:
        (sp,) = s.sort_windows(win)
    r = ko.sort_window(win.T, oss, max_iters=50)
    nt, nt0 = oss.wPCA.shape[1], oss.nt0min
    a, amp_ok, amax = agreement(r.match.st[:, 0] - nt // 2 + nt0, r.match.st[:, 1], r.match.amps,
                                sp["time"], sp["tmpl"], sp["amp"])
    assert len(r.match.st) > 800
    assert a >= AGREE and amp_ok >= AGREE, (a, amp_ok, amax, len(sp), len(r.match.st))


def test_pruned_tier_lists_in_global_memory(cfg_small):
    """A 60000-sample window keeps its lists in global memory: same bar against the full loop,
    and a rerun is bitwise identical."""
    d, data, _ = cfg_small
    win = data[: 60000 + 122]
    outs = {}
    for keep in (0, 32):
        with sorter.OnlineSorter(d, max_iters=50, match_keep=keep) as s:
            outs[keep] = s.sort_windows(win)[0]
            if keep:
                again = s.sort_windows(win)[0]
    a, amp_ok, amax = agreement(outs[0]["time"], outs[0]["tmpl"], outs[0]["amp"],
                                outs[32]["time"], outs[32]["tmpl"], outs[32]["amp"])
    assert len(outs[0]) > 500
    assert a >= AGREE and amp_ok >= AGREE, (a, amp_ok, amax)
    for f in ("time", "tmpl", "amp", "pcfeat"):
        np.testing.assert_array_equal(again[f], outs[32][f])


def test_match_keep_is_validated(golden_dir, tmp_path):
    z = np.load(golden_dir / "ks_window.npz")
    d = write_oss_from_arrays(z, tmp_path / "oss_input")
    with pytest.raises(sorter.SorterError) as e:
        sorter.OnlineSorter(d, match_keep=33)
    assert e.value.status == 1
    for bad in (dict(match_keep=16, match_keep_wide=16), dict(match_keep=16, match_keep_wide=33),
                dict(match_keep=0, match_keep_wide=24), dict(match_keep=16, match_keep_wide=24, match_keep_crowd=-1.0)):
        with pytest.raises(sorter.SorterError) as e:
            sorter.OnlineSorter(d, **bad)
        assert e.value.status == 1, bad
