"""The low-precision projection tiers against the float64 oracle (Kilosort's loop on exact scores):
gemm_path 4 = one BF16 product, gemm_path 5 = one FP8 e4m3 product with per-(component, channel)
and per-template scales; both accumulate in FP32 and recompute every accepted candidate's amplitude
from the exact FP32 projection of the split operands.  The scores differ from FP32 by the
products' rounding (bounded below), and spikes differ where that rounding ranks candidates
differently, so the agreement is measured per config and bounded here at its measured level:

  config                                   BF16 x1: spikes / amplitudes   FP8 e4m3: spikes / amplitudes
  384 ch, 500 templates, 10 Hz stream      >= 99.5 % / >= 99.5 %          >= 98.5 % / >= 94 %
  128 ch, 200 templates, 30 Hz, overlaps   >= 99.5 % / >= 99.5 %          >= 97.5 % / >= 88 %
  384 ch, 500 templates, 40 Hz stream      >= 98.5 % / >= 99.5 %          >= 94.5 % / >= 90 %

(amplitudes: the fraction of matched spikes within 1e-3 relative).  Only the BF16 tier meets the
99.5 % bar, and only below 40 Hz; the FP8 tier does not at any rate."""
import numpy as np
import pytest

from livespikesorter_gb300 import sorter, synth
from oracle import ks_oracle as ko

from lss_testutil import agreement, make_dataset

pytestmark = pytest.mark.gpu

BOUNDS = {  # (gemm_path, config) -> (spikes, amplitudes)
    (4, "stream"): (0.995, 0.995), (4, "dense"): (0.995, 0.995), (4, "stream40"): (0.985, 0.995),
    (5, "stream"): (0.985, 0.94), (5, "dense"): (0.975, 0.88), (5, "stream40"): (0.945, 0.90),
}
SCORE_ERR = {4: 4e-3, 5: 4e-2}   # largest score error over the largest score magnitude


@pytest.fixture(scope="module")
def cfg_stream40(tmp_path_factory):
    cfg = synth.SynthConfig(n_chan=384, n_units=500, n_samples=6 * 1500 + 300, drift_um=20.0, whiten_batch=3000,
                            whiten_batches=3, seed=7, rate_hz=40.0)
    return make_dataset(cfg, tmp_path_factory.mktemp("cfg2_40hz"))


def _reference(name, d, data):
    oss = ko.load_oss_input(d)
    if name == "dense":
        win = data[: 12000 + 122]
        r = ko.sort_window(win.T, oss, max_iters=50)
        return (r.match.st[:, 0] - oss.wPCA.shape[1] // 2 + oss.nt0min, r.match.st[:, 1], r.match.amps), win
    rr = ko.sort_stream(data, oss, 1500, max_iters=50)
    k = rr["keep"]
    return (rr["time"][k], rr["template"][k], rr["amp"][k]), data[:1622]


@pytest.mark.parametrize("gemm_path", [4, 5])
@pytest.mark.parametrize("name", ["stream", "dense", "stream40"])
def test_low_precision_tier_vs_float64(name, gemm_path, cfg_stream, cfg_dense, cfg_stream40):
    d, data, _ = {"stream": cfg_stream, "dense": cfg_dense, "stream40": cfg_stream40}[name]
    ref, win = _reference(name, d, data)
    with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=4) as s0:
        exact = s0.debug_stage(win, sorter.STAGE_SCORES).astype(np.float64)
    with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=4, gemm_path=gemm_path) as s:
        sp = s.sort_windows(win)[0] if name == "dense" else s.sort_stream(data)
        scores = s.debug_stage(win, sorter.STAGE_SCORES).astype(np.float64)
    err = np.abs(scores - exact).max() / np.abs(exact).max()
    assert err <= SCORE_ERR[gemm_path], err
    a, amp_ok, amax = agreement(ref[0], ref[1], ref[2], sp["time"], sp["tmpl"], sp["amp"])
    want_a, want_amp = BOUNDS[(gemm_path, name)]
    assert len(ref[0]) > 300
    assert a >= want_a and amp_ok >= want_amp, (a, amp_ok, amax, len(sp), len(ref[0]))


def test_low_precision_tiers_are_deterministic_and_validated(cfg_stream, tmp_path):
    d, data, _ = cfg_stream
    runs = []
    for _ in range(2):
        with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=4, gemm_path=5) as s:
            runs.append(s.sort_stream(data))
    for f in ("time", "tmpl", "amp"):
        np.testing.assert_array_equal(runs[0][f], runs[1][f])
    with pytest.raises(sorter.SorterError):
        sorter.OnlineSorter(d, batch_samples=1500, gemm_path=5, match_keep=16)
    with pytest.raises(sorter.SorterError):
        sorter.OnlineSorter(d, batch_samples=1500, gemm_path=6)
