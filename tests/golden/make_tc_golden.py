"""Generate tests/golden/tc_reference.npz by running the reference's own threshold-crossing sorter
(src/SpikeSorter/ThresholdCrossing.cpp, compiled unmodified by oracle/build_ref.py under stubs for
its socket / SDK types) on a scripted replay of seeded int16 rows.

The rows are regenerated by ``rows()`` from the stored seed (numpy's default_rng is the same on
every platform), so the fixture holds only the replay schedule, the calibration the reference
code has compiled in (its per-channel means and medians, read from the source as text) and the
events of every payload it sent: the stream count it stamped (its lLatestCt) and the (time,
channel) pairs in emission order.

    python tests/golden/make_tc_golden.py            (needs the reference checkout)
"""
from __future__ import annotations

import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
C, N, SEED = 64, 6000, 17
MIN_WINDOW, MAX_WINDOW, THRESHOLD_STD = 300, 2500, 4.0
# stream counts the replay socket reports, one per wait: regular batches, a jump past the maximum
# window (the reference then fetches only the newest MAX_WINDOW rows) and a batch the minimum
# window skips
SCHEDULE = [2500, 2800, 3250, 3600, 5900, 5950, 6000]


def reference_calibration(src: Path):
    """The per-channel means and medians compiled into ThresholdCrossing.cpp (the uncommented
    ``std::vector<float> means / medians = {...}`` lines)."""
    text = src.read_text()
    out = {}
    for name in ("means", "medians"):
        m = re.search(r"^\s*std::vector<float> " + name + r" = \{([^}]*)\};", text, re.M)
        out[name] = np.array([float(v) for v in m.group(1).split(",") if v.strip()], np.float32)
    return out["means"], out["medians"]


def rows(means, medians, seed=SEED, n=N, c=C):
    """Seeded int16 rows around the compiled-in means: noise of each channel's median scale,
    negative spikes, and values on each channel's threshold boundary (and one either side)."""
    rng = np.random.default_rng(seed)
    mu, md = means[:c].astype(np.float64), np.maximum(medians[:c].astype(np.float64), 1.0)
    x = mu[None, :] + rng.normal(0, 1, (n, c)) * 1.4 * md[None, :]
    for _ in range(n * c // 400):
        t, ch = rng.integers(0, n - 10), rng.integers(0, c)
        x[t:t + 6, ch] -= rng.uniform(3, 9) * md[ch] * np.hanning(6)
    xi = np.clip(np.round(x), -32768, 32767).astype(np.int16)
    # the threshold boundary: the largest int16 v with (float)v - mean <= -thr * median (in double)
    for ch in range(c):
        lim = -1.0 * np.float64(np.float32(THRESHOLD_STD)) * np.float64(np.float32(medians[ch]))
        v = np.arange(-2000, 2000, dtype=np.int32)
        ok = (v.astype(np.float32) - np.float32(means[ch])).astype(np.float64) <= lim
        b = int(v[ok].max())
        for k, d in enumerate((-1, 0, 1)):
            xi[100 + 37 * ch % (n - 200) + k, ch] = b + d
    return xi


def main():
    sys.path.insert(0, str(ROOT))
    from oracle import build_ref
    exe = build_ref.build_tc(verbose=True)
    if exe is None:
        raise SystemExit("the reference checkout is needed to run its threshold-crossing code")
    means, medians = reference_calibration(build_ref.REFERENCE / "src" / "SpikeSorter" / "ThresholdCrossing.cpp")
    x = rows(means, medians)
    with tempfile.TemporaryDirectory() as td:
        x.tofile(Path(td) / "rows.bin")
        r = subprocess.run([str(exe), str(Path(td) / "rows.bin"), str(C), str(MIN_WINDOW), str(MAX_WINDOW),
                            str(THRESHOLD_STD)] + [str(s) for s in SCHEDULE], capture_output=True, text=True,
                           check=True, cwd=td)
    lines = r.stdout.splitlines()
    latest, counts, times, chans = [], [], [], []
    i = 0
    while i < len(lines):
        lat, n = map(int, lines[i].split())
        latest.append(lat)
        counts.append(n)
        for ln in lines[i + 1:i + 1 + n]:
            t, ch = ln.split(",")
            times.append(int(t))
            chans.append(int(ch))
        i += 1 + n
    np.savez_compressed(HERE / "tc_reference.npz", seed=SEED, C=C, N=N, min_window=MIN_WINDOW,
                        max_window=MAX_WINDOW, threshold_std=np.float32(THRESHOLD_STD),
                        schedule=np.array(SCHEDULE, np.int64), means=means, medians=medians,
                        latest=np.array(latest, np.int64), counts=np.array(counts, np.int64),
                        times=np.array(times, np.int64), channels=np.array(chans, np.int32))
    print(f"{len(latest)} payloads, {len(times)} events -> {HERE / 'tc_reference.npz'}")


if __name__ == "__main__":
    main()
