"""The threshold-crossing oracle pinned against the reference's own code: tests/golden/
tc_reference.npz holds the events that src/SpikeSorter/ThresholdCrossing.cpp emitted when compiled
unmodified under stubs (oracle/build_ref.py, tests/golden/make_tc_golden.py) and run on a scripted
replay of seeded int16 rows -- regular batches, a jump past the maximum window, a batch the
minimum window skips, values on every channel's threshold boundary.  The restatement
(oracle/tc_oracle.py) reproduces every payload's events, in the reference's order, with the
reference's calibration; the reference stamps row r of a fetch with its lLatestCt + r
(ThresholdCrossing.cpp:207,224), the newest stream count, which the check applies too."""
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import tc_oracle

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import make_tc_golden as mk  # noqa: E402


@pytest.fixture(scope="module")
def ref():
    return np.load(GOLDEN / "tc_reference.npz")


def fetches(z):
    """(latest, first row, last row) of each batch the reference processed: it waits for
    processed + min_window, reads the stream count and fetches [processed, latest), at most the
    newest max_window rows (ThresholdCrossing.cpp:186-207, dataSocket.cpp:128-153)."""
    sched = [int(v) for v in z["schedule"]]
    mn, mx = int(z["min_window"]), int(z["max_window"])
    at, processed, out = 0, sched[0], []
    while True:
        while sched[at] < processed + mn:
            at += 1
            if at >= len(sched):
                return out
        latest = sched[at]
        start = latest - mx if latest - processed > mx else processed
        out.append((latest, start, latest))
        processed = latest


def test_oracle_reproduces_the_reference_run(ref):
    C = int(ref["C"])
    x = mk.rows(ref["means"], ref["medians"], int(ref["seed"]), int(ref["N"]), C)
    fs = fetches(ref)
    assert [f[0] for f in fs] == list(ref["latest"])
    off = 0
    for (latest, a, b), n in zip(fs, ref["counts"]):
        t, c, _ = tc_oracle.threshold_crossings(x[a:b], ref["means"][:C], ref["medians"][:C],
                                                float(ref["threshold_std"]), first_row_sample=latest)
        np.testing.assert_array_equal(t, ref["times"][off:off + n])
        np.testing.assert_array_equal(c, ref["channels"][off:off + n])
        off += int(n)
    assert off == len(ref["times"]) > 1000


def test_boundary_values_are_in_the_fixture(ref):
    """The rows carry each channel's boundary value: the reference fired on it, not on the value
    above."""
    C = int(ref["C"])
    x = mk.rows(ref["means"], ref["medians"], int(ref["seed"]), int(ref["N"]), C)
    lim = tc_oracle.limits(ref["medians"][:C], float(ref["threshold_std"]))
    y = (x.astype(np.float32) - ref["means"][:C].astype(np.float32)).astype(np.float64)
    at_boundary = np.isclose(y, lim[None, :], atol=1.0) & (y <= lim[None, :])
    assert at_boundary.sum() >= C
