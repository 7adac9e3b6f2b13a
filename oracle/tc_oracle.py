"""ORACLE -- test infrastructure, not product code.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs may import this module, and only as the checker.

CPU restatement of the reference's threshold-crossing sorter
(src/SpikeSorter/ThresholdCrossing.cpp, class ThresholdCrossing), in numpy.

Parity: pinned against the reference's own code.  oracle/build_ref.py compiles the reference's
src/SpikeSorter/ThresholdCrossing.cpp unmodified under stubs for its socket / SDK / networking
types, tests/golden/make_tc_golden.py runs it on a scripted replay of seeded int16 rows, and
tests/test_tc_reference_cpu.py checks that this restatement reproduces every payload's events in
order (tests/golden/tc_reference.npz).  Each function cites the lines it follows.

Semantics restated:
  * DC removal in float32: ``m_fY[j] = m_fY[j] - means[i]`` (ThresholdCrossing.cpp:210-214), the
    rows being int16 converted to float exactly (StreamDataSocket::fetchLatest_TC,
    dataSocket.cpp:146-148);
  * the test ``m_fY[j] <= -1.0 * m_fThresholdStd * medians[i]`` (ThresholdCrossing.cpp:223), which
    C++ evaluates in double (the literal -1.0 is a double);
  * emission order: channel by channel, rows in order within a channel (the loops of
    ThresholdCrossing.cpp:218-230), template = channel, amplitude 0;
  * calibration as the commented-out code computes it (ThresholdCrossing.cpp:146-177): per-channel
    mean, then the element at index n/2 of the sorted absolute mean-removed samples.
Deliberate difference: times are ``first_row_sample + row``; the reference adds the row to the
stream count read before the fetch (ThresholdCrossing.cpp:207,224), the newest sample of the
fetch, which is not restated.
"""
from __future__ import annotations

import numpy as np


def mean_removed(rows, means):
    """float32 ``(float)x - means[c]`` (ThresholdCrossing.cpp:210-214)."""
    return np.asarray(rows).astype(np.float32) - np.asarray(means, np.float32)[None, :]


def limits(medians, threshold_std):
    """``-1.0 * m_fThresholdStd * medians[i]`` in double (ThresholdCrossing.cpp:223)."""
    with np.errstate(invalid="ignore", over="ignore"):
        return -1.0 * np.float64(np.float32(threshold_std)) * np.asarray(medians, np.float32).astype(np.float64)


def threshold_crossings(rows, means, medians, threshold_std, first_row_sample=0):
    """Events of one fetched block of rows [n][C] int16, in the reference's order
    (ThresholdCrossing.cpp:218-230): returns (time int64, channel int32, value float32)."""
    rows = np.asarray(rows)
    if rows.size == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int32), np.zeros(0, np.float32)
    with np.errstate(invalid="ignore", over="ignore"):
        y = mean_removed(rows, means)
        hit = y.astype(np.float64) <= limits(medians, threshold_std)[None, :]
    ch, r = np.nonzero(hit.T)                 # channel-major, rows ascending within a channel
    return (np.int64(first_row_sample) + r.astype(np.int64), ch.astype(np.int32), y[r, ch])


def int_thresholds(means, medians, threshold_std):
    """Largest int16 x whose test passes, per channel (-32769 when none): the integer form of
    ThresholdCrossing.cpp:223, found by evaluating the float test on every int16 value."""
    x = np.arange(-32768, 32768, dtype=np.int32)
    xf = x.astype(np.float32)
    lim = limits(medians, threshold_std)
    out = np.empty(len(lim), np.int32)
    for c, m in enumerate(np.asarray(means, np.float32)):
        with np.errstate(invalid="ignore", over="ignore"):
            hit = (xf - m).astype(np.float64) <= lim[c]
        idx = np.nonzero(hit)[0]
        out[c] = x[idx[-1]] if idx.size else -32769
    return out


def calibrate(rows):
    """Per-channel (means, medians) of a block of rows as ThresholdCrossing.cpp:146-177 computes
    them: mean = (float)sum / (float)n (sum exact in int64), median = element n//2 of the sorted
    |(float)x - mean|."""
    rows = np.asarray(rows)
    n = rows.shape[0]
    sums = rows.astype(np.int64).sum(0)
    means = (sums.astype(np.float32) / np.float32(n)).astype(np.float32)
    dev = np.abs(rows.astype(np.float32) - means[None, :])
    medians = np.sort(dev, axis=0)[n // 2].astype(np.float32)
    return means, medians


def sort_blocks(rows, blocks, means, medians, threshold_std, first_row_sample=0):
    """The events of a stream cut into consecutive fetches of the given lengths, block by block
    (the loop of ThresholdCrossing.cpp:195-252 with each fetch's own start)."""
    out_t, out_c, out_v = [], [], []
    s = 0
    for n in blocks:
        t, c, v = threshold_crossings(rows[s:s + n], means, medians, threshold_std, first_row_sample + s)
        out_t.append(t)
        out_c.append(c)
        out_v.append(v)
        s += n
    if not out_t:
        return np.zeros(0, np.int64), np.zeros(0, np.int32), np.zeros(0, np.float32)
    return np.concatenate(out_t), np.concatenate(out_c), np.concatenate(out_v)
