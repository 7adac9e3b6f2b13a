"""Threshold-crossing detector, host side (no GPU): the integer thresholds and the calibration of
the C library against the oracle's restatement of ThresholdCrossing.cpp, the integer form of the
test against the float/double test itself, the C struct layout, and argument errors."""
import ctypes as ct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from livespikesorter_gb300 import sorter, threshold
from oracle import tc_oracle

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    return sorter.load_library()


def _stats(rng, C):
    means = (rng.normal(0, 20, C)).astype(np.float32)
    medians = rng.integers(1, 10, C).astype(np.float32)
    return means, medians


def test_int_thresholds_match_oracle(lib):
    rng = np.random.default_rng(11)
    means, medians = _stats(rng, 64)
    # awkward values: integers, halves, tiny, huge, zero / negative medians, non-finite
    means[:12] = [0.0, 0.5, -0.5, 3.0, -7.25, 1e-7, -1e-7, 4e4, -4e4, np.nan, np.inf, -np.inf]
    medians[12:20] = [0.0, -2.0, 0.1, 1e-3, 3e4, np.nan, np.inf, 123.456]
    for thr in (3.0, 3.3, 4.5, 0.0, -1.0):
        got = threshold.int_thresholds(means, medians, thr)
        want = tc_oracle.int_thresholds(means, medians, thr)
        np.testing.assert_array_equal(got, want, err_msg=f"threshold_std={thr}")


def test_float_double_boundary_follows_double():
    """A sample whose float value equals the float32-rounded limit but lies above the exact
    double limit (ThresholdCrossing.cpp:223 compares in double) must not cross."""
    thr, med = np.float32(3.3), np.float32(3.0)
    lim = -1.0 * np.float64(thr) * np.float64(med)
    lim_f = np.float32(np.float32(thr) * np.float32(med))
    assert np.float64(lim_f) < -lim                       # float rounding of the product went down
    # a mean that puts x = -10 exactly on the float limit
    found = None
    for m in np.arange(-0.2, 0.0, 1e-6, dtype=np.float64).astype(np.float32):
        if np.float32(np.float32(-10) - m) == -lim_f:
            found = m
            break
    assert found is not None
    rows = np.array([[-10], [-11], [-9]], np.int16)
    t, c, v = tc_oracle.threshold_crossings(rows, [found], [med], thr)
    assert list(t) == [1]                                 # -11 crosses, -10 sits above the double limit
    X = threshold.int_thresholds(np.array([found], np.float32), np.array([med], np.float32), float(thr))
    assert X[0] == -11


def test_integer_form_equals_reference_test():
    """x <= X[c] selects exactly the samples the reference's test selects, in its order."""
    rng = np.random.default_rng(5)
    C, n = 48, 3000
    means, medians = _stats(rng, C)
    rows = rng.normal(0, 12, (n, C)).astype(np.int16)
    rows[rng.integers(0, n, 40), rng.integers(0, C, 40)] = -200
    for thr in (2.0, 3.0, 4.0):
        t, c, v = tc_oracle.threshold_crossings(rows, means, medians, thr, first_row_sample=1000)
        X = threshold.int_thresholds(means, medians, thr)
        ch, r = np.nonzero((rows.astype(np.int32) <= X[None, :]).T)
        np.testing.assert_array_equal(t, 1000 + r)
        np.testing.assert_array_equal(c, ch)
        np.testing.assert_array_equal(v, rows[r, ch].astype(np.float32) - means[ch])
        assert len(t) > 0


def test_calibrate_matches_oracle():
    rng = np.random.default_rng(2)
    for n, C in ((1, 3), (2, 5), (1001, 40), (4000, 17)):
        rows = (rng.normal(0, 15, (n, C)) + rng.normal(0, 30, C)).astype(np.int16)
        mu, md = threshold.calibrate(rows)
        mu_o, md_o = tc_oracle.calibrate(rows)
        np.testing.assert_array_equal(mu, mu_o)
        np.testing.assert_array_equal(md, md_o)


def test_sort_blocks_is_blockwise():
    rng = np.random.default_rng(8)
    rows = rng.normal(0, 10, (500, 8)).astype(np.int16)
    means, medians = _stats(rng, 8)
    t, c, v = tc_oracle.sort_blocks(rows, [100, 0, 250, 150], means, medians, 2.0, first_row_sample=7)
    parts = [tc_oracle.threshold_crossings(rows[a:b], means, medians, 2.0, 7 + a)
             for a, b in ((0, 100), (100, 350), (350, 500))]
    np.testing.assert_array_equal(t, np.concatenate([p[0] for p in parts]))
    np.testing.assert_array_equal(c, np.concatenate([p[1] for p in parts]))


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "tc.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "lss_threshold.h"\n'
                   'int main(){printf("%zu %zu %zu %zu %zu\\n", sizeof(lss_tc_params), sizeof(lss_tc_event),'
                   ' offsetof(lss_tc_params, max_rows), offsetof(lss_tc_params, profile),'
                   ' offsetof(lss_tc_event, value));return 0;}\n')
    exe = tmp_path / "tc"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [ct.sizeof(threshold.TcParams), ct.sizeof(threshold.TcEvent), threshold.TcParams.max_rows.offset,
                   threshold.TcParams.profile.offset, threshold.TcEvent.value.offset]


def test_default_params(lib):
    p = threshold.TcParams()
    assert lib.lss_tc_default_params(ct.byref(p)) == 0
    assert (p.abi_version, p.threshold_std, p.max_rows, p.event_cap) == (1, 3.0, 1500, 0)
    assert lib.lss_tc_default_params(None) == 1


def test_bad_open_arguments(lib):
    mu = np.zeros(8, np.float32)
    md = np.ones(8, np.float32)
    h = ct.c_void_p()
    for field, value, word in (("n_chan", 0, "n_chan"), ("n_chan", 5000, "n_chan"), ("n_chan", 515, "multiple of 8"),
                               ("max_rows", 0, "max_rows"), ("max_rows", 1 << 30, "2^31"),
                               ("abi_version", 9, "abi_version")):
        p = threshold.TcParams()
        lib.lss_tc_default_params(ct.byref(p))
        p.n_chan = 8
        setattr(p, field, value)
        big_mu = np.zeros(max(8, p.n_chan), np.float32)
        big_md = np.ones(max(8, p.n_chan), np.float32)
        st = lib.lss_tc_open(ct.byref(p), big_mu.ctypes.data, big_md.ctypes.data, ct.byref(h))
        assert st == 1, (field, value, st)
        assert word in lib.lss_tc_last_error(None).decode()
    p = threshold.TcParams()
    lib.lss_tc_default_params(ct.byref(p))
    p.n_chan = 8
    assert lib.lss_tc_open(ct.byref(p), None, md.ctypes.data, ct.byref(h)) == 1
    assert lib.lss_tc_open(ct.byref(p), mu.ctypes.data, md.ctypes.data, None) == 1


def test_null_handles_rejected(lib):
    n = ct.c_int64()
    assert lib.lss_tc_push(None, None, 0, 0) == 1
    assert lib.lss_tc_poll(None, None, 0, ct.byref(n)) == 1
    assert lib.lss_tc_pending(None, ct.byref(n)) == 1
    assert lib.lss_tc_close(None) == 1
    assert lib.lss_tc_int_thresholds(-1, None, None, ct.c_float(3.0), None) == 1
    assert lib.lss_tc_calibrate(None, 0, 0, None, None) == 1


def test_no_gpu_open_fails_cleanly(lib):
    pytest.importorskip("torch")
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(sorter.SorterError) as e:
        threshold.ThresholdCrossing(np.zeros(16), np.ones(16), 3.0)
    assert e.value.status == 4
