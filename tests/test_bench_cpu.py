"""bench.py's host-side arithmetic without a GPU: the roofline line of each possible dominant
kernel (algorithmic work per launch over its duration, against the measured peaks), the DRAM side
of the matching loop, and the spike-agreement rule used for the faster tier and the proposal gate."""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
from livespikesorter_gb300 import sorter  # noqa: E402

SHAPE = dict(C=384, T=500, K=6, nt=61, W=1622, ntaps=885, spikes_per_batch=230.0)


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops_sustained", 1700.0)
    return 6800.0, 1700.0


def test_roofline_of_the_matching_loop():
    stages = {"h2d": 99.0, "car": 0.31, "highpass": 0.40, "whiten": 0.29, "basis_conv": 0.54, "project": 0.84,
              "match": 2.09, "features": 0.10, "d2h": 99.0}
    n = 4
    r = bench.roofline({k: v * n for k, v in stages.items()}, n, 64, **SHAPE)
    hbm, _ = _peaks()
    assert r["kernel"] == "match" and r["bound"] == "hbm" and r["unit"] == "GB/s"   # h2d / d2h never chosen
    C, T, nt, W = SHAPE["C"], SHAPE["T"], SHAPE["nt"], SHAPE["W"]
    per_spike = T * (2 * nt + 1) * 12   # ctc read + score read-modify-write; no residual on the sorting path
    bytes_ = 64 * (4 * T * W + SHAPE["spikes_per_batch"] * per_spike)
    assert r["achieved"] == pytest.approx(bytes_ / 1e9 / 2.09e-3)
    assert r["frac"] == pytest.approx(r["achieved"] / hbm)
    assert r["traffic"] == pytest.approx(8.477e9)
    assert r["dram_gbs"] == pytest.approx(r["traffic"] / 1e9 / 2.09e-3)
    assert r["dram_frac"] < r["frac"] and "note" in r          # L2 reuse: algorithmic bytes above DRAM


@pytest.mark.parametrize("kern,flop", [
    ("project", lambda s: 2 * s["T"] * s["K"] * s["C"] * s["W"]),
    ("highpass", lambda s: 2 * s["C"] * s["W"] * s["ntaps"]),
    ("whiten", lambda s: 2 * s["C"] ** 2 * s["W"]),
    ("basis_conv", lambda s: 2 * s["C"] * s["K"] * s["nt"] * s["W"]),
])
def test_roofline_of_the_tensor_core_stages(kern, flop):
    stages = {"match": 0.1, kern: 1.0}
    r = bench.roofline(stages, 1, 8, **SHAPE)
    _, tf = _peaks()
    assert r["kernel"] == kern and r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert r["achieved"] == pytest.approx(8 * flop(SHAPE) / 1e12 / 1e-3)
    assert r["frac"] == pytest.approx(r["achieved"] / tf)
    assert "dram_gbs" not in r


def _spikes(t, k, a):
    s = np.zeros(len(t), sorter.SPIKE_DTYPE)
    s["time"], s["tmpl"], s["amp"] = t, k, a
    return s


def test_spike_agreement_rule():
    ref = _spikes([100, 200, 300, 400], [1, 2, 3, 4], [10.0, 20.0, 30.0, 40.0])
    got = _spikes([101, 200, 300, 405, 500], [1, 2, 9, 4, 5], [10.0, 20.00001, 30.0, 40.0, 1.0])
    frac, amp_ok = bench.spike_agreement(ref, got)
    # 100 matches 101 (|dt| = 1), 200 exact; 300 has the wrong template, 400 is 5 samples off
    assert frac == pytest.approx(0.5) and amp_ok == pytest.approx(1.0)
    frac, amp_ok = bench.spike_agreement(ref, _spikes([100, 100], [1, 1], [10.0, 10.5]))
    assert frac == pytest.approx(0.25) and amp_ok == pytest.approx(1.0)   # each got spike used once
    assert bench.spike_agreement(ref[:0], got) == (1.0, 1.0)
    frac, amp_ok = bench.spike_agreement(ref[:1], _spikes([100], [1], [10.02]))
    assert frac == 1.0 and amp_ok == 0.0                                     # 2e-3 relative: outside 1e-3
