"""Threshold-crossing detector on the GPU, through the C ABI (include/lss_threshold.h): every
event equal to the oracle's restatement of ThresholdCrossing.cpp -- time, channel, value bit for
bit and in the reference's order -- over channel counts that take the vector and the scalar
kernels, pushes of one sample up to a long recording, units whose crossings overflow the kept
list, the event cap, device-resident input, and the C++ drop-in class."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from livespikesorter_gb300 import sorter, threshold
from oracle import tc_oracle

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    sorter.load_library()


def recording(n, C, seed, rate_hz=40.0, fs=30000.0):
    """Seeded int16 rows: per-channel DC offset and Gaussian noise, plus negative biphasic spikes
    spread over a few neighbouring channels."""
    rng = np.random.default_rng(seed)
    dc = rng.normal(0, 20, C)
    sd = rng.uniform(5, 12, C)
    x = rng.normal(0, 1, (n, C)) * sd[None, :] + dc[None, :]
    n_sp = rng.poisson(rate_hz * C / 8 * n / fs)
    t0 = rng.integers(0, max(1, n - 40), n_sp)
    c0 = rng.integers(0, C, n_sp)
    amp = rng.lognormal(np.log(90), 0.4, n_sp)
    wave = -np.exp(-0.5 * ((np.arange(30) - 10) / 2.5) ** 2) + 0.35 * np.exp(-0.5 * ((np.arange(30) - 18) / 4) ** 2)
    for t, c, a in zip(t0, c0, amp):
        for dcn in range(-2, 3):
            cc = c + dcn
            if 0 <= cc < C:
                seg = x[t:t + 30, cc]
                seg += a * np.exp(-0.5 * dcn * dcn) * wave[:len(seg)]
    return np.clip(np.round(x), -32768, 32767).astype(np.int16)


def expect(rows, means, medians, thr, first=0):
    t, c, v = tc_oracle.threshold_crossings(rows, means, medians, thr, first)
    return t, c, v


def assert_events_equal(ev, t, c, v):
    assert len(ev) == len(t), (len(ev), len(t))
    np.testing.assert_array_equal(ev["time"], t)
    np.testing.assert_array_equal(ev["channel"], c)
    np.testing.assert_array_equal(ev["value"].view(np.uint32), v.astype(np.float32).view(np.uint32))


@pytest.mark.parametrize("C,n,thr", [(384, 1500, 3.0), (384, 1500, 4.5), (32, 4096, 3.0), (30, 1500, 3.0),
                                     (1, 700, 2.5), (512, 333, 3.0), (4096, 600, 3.0)])
def test_pushes_match_oracle(C, n, thr):
    rows = recording(n * 3, C, seed=C + n)
    means, medians = tc_oracle.calibrate(rows[:n])
    with threshold.ThresholdCrossing(means, medians, thr, max_rows=n) as tc:
        np.testing.assert_array_equal(tc.thresholds(), tc_oracle.int_thresholds(means, medians, thr))
        blocks = [n, 1, n - 1, n]
        s = 0
        for b in blocks:
            tc.push(rows[s:s + b], first_row_sample=10_000 + s)
            s += b
            assert tc.kernel_launches() == 4
        ev = tc.poll_all()
    t, c, v = tc_oracle.sort_blocks(rows, blocks, means, medians, thr, first_row_sample=10_000)
    assert len(t) > 0
    assert_events_equal(ev, t, c, v)


def test_long_recording_single_push():
    """One push of 200k rows x 384 channels (153 MB, larger than L2; slab length grows)."""
    C, n = 384, 200_000
    rows = recording(n, C, seed=99)
    means, medians = tc_oracle.calibrate(rows[:30000])
    with threshold.ThresholdCrossing(means, medians, 3.0, max_rows=n) as tc:
        tc.push(rows, first_row_sample=5)
        ev = tc.poll_all()
    assert_events_equal(ev, *expect(rows, means, medians, 3.0, 5))


def test_dense_units_reread_rows():
    """Channels below threshold for hundreds of consecutive rows: units keep 32 crossings and
    must read their rows again to place the rest."""
    C, n = 64, 5000
    rows = recording(n, C, seed=4)
    means, medians = tc_oracle.calibrate(rows)
    rows[1000:1700, 8:16] = -3000      # one channel group, long run
    rows[2000:2003, :] = -3000         # every channel, short run
    rows[4990:, 63] = -3000            # tail of the last slab
    with threshold.ThresholdCrossing(means, medians, 3.0, max_rows=n) as tc:
        tc.push(rows, first_row_sample=0)
        ev = tc.poll_all()
    t, c, v = expect(rows, means, medians, 3.0)
    assert (c == 8).sum() >= 700
    assert_events_equal(ev, t, c, v)


def test_event_cap_overflow_keeps_first_events():
    C, n = 64, 2000
    rows = recording(n, C, seed=6)
    means, medians = tc_oracle.calibrate(rows)
    rows[:200, :] = -3000
    t, c, v = expect(rows, means, medians, 3.0)
    cap = 4096
    assert len(t) > cap
    with threshold.ThresholdCrossing(means, medians, 3.0, max_rows=n, event_cap=cap) as tc:
        tc.push(rows)
        ev, st = tc.poll(cap=100_000, allow_overflow=True)
        assert st == 6
        ev2, st2 = tc.poll(cap=10, allow_overflow=True)
        assert st2 == 0 and len(ev2) == 0
    assert_events_equal(ev, t[:cap], c[:cap], v[:cap])


def test_empty_and_oversized_pushes():
    means, medians = np.zeros(16, np.float32), np.ones(16, np.float32)
    with threshold.ThresholdCrossing(means, medians, 3.0, max_rows=100) as tc:
        tc.push(np.zeros((0, 16), np.int16))
        assert tc.kernel_launches() == 0
        assert len(tc.poll_all()) == 0
        with pytest.raises(sorter.SorterError) as e:
            tc.push(np.zeros((101, 16), np.int16))
        assert e.value.status == 1
        rows = np.full((100, 16), -5, np.int16)
        tc.push(rows, first_row_sample=3)
        ev = tc.poll_all()
    assert_events_equal(ev, *expect(rows, means, medians, 3.0, 3))


def test_device_rows_aligned_and_unaligned():
    torch = pytest.importorskip("torch")
    C, n = 96, 3000
    rows = recording(n + 1, C, seed=12)
    means, medians = tc_oracle.calibrate(rows)
    d = torch.from_numpy(rows.reshape(-1).copy()).cuda()
    with threshold.ThresholdCrossing(means, medians, 3.0, max_rows=n) as tc:
        torch.cuda.synchronize()
        tc.push_device(d.data_ptr(), n, first_row_sample=0)                    # 16-byte aligned: 8 channels a thread
        tc.push_device(d.data_ptr() + 2 * C, n, first_row_sample=1)            # next row: still aligned (C*2 = 192 B)
        tc.push_device(d[C + 1:].data_ptr(), 1, first_row_sample=77)           # 2-byte offset: one channel a thread
        ev = tc.poll_all()
        torch.cuda.synchronize()
    r_un = rows.reshape(-1)[C + 1:C + 1 + C].reshape(1, C)
    parts = [expect(rows[:n], means, medians, 3.0, 0), expect(rows[1:n + 1], means, medians, 3.0, 1),
             expect(r_un, means, medians, 3.0, 77)]
    assert_events_equal(ev, *(np.concatenate([p[i] for p in parts]) for i in range(3)))


def test_stage_times_and_streams():
    C, n = 384, 1500
    rows = recording(n * 4, C, seed=21)
    means, medians = tc_oracle.calibrate(rows)
    with threshold.ThresholdCrossing(means, medians, 3.0, max_rows=n, profile=1) as tc:
        for i in range(4):
            tc.push(rows[i * n:(i + 1) * n], first_row_sample=i * n)
        ev = tc.poll_all()
        ms, k = tc.stage_times()
        assert k == 4 and all(v >= 0 for v in ms.values()) and ms["count"] > 0
        assert tc.cuda_stream() != 0
    assert_events_equal(ev, *tc_oracle.sort_blocks(rows, [n] * 4, means, medians, 3.0))


def replay_blocks(n, tick, max_window):
    """(start, length) of each fetch lss::ThresholdCrossing makes from the example's replay socket
    (which reports the rows available so far, then makes tick more arrive): the newest max_window
    rows when more than that arrived (dataSocket.cpp:128-154)."""
    avail = 0

    def query():
        nonlocal avail
        now = avail
        avail = min(n, avail + tick)
        return now

    processed = query()
    fetched = 0
    out = []
    while True:
        latest = query()
        if latest <= processed:
            if fetched >= n:
                break
            continue
        start = max(processed, avail - max_window if avail > max_window else 0)
        end = min(avail, start + max_window)
        if end <= processed:
            if fetched >= n:
                break
            continue
        fetched = max(fetched, end)
        m = min(end - processed, max_window)
        out.append((end - m, m))
        processed = end
    return out


def test_cpp_threshold_crossing_replay(tmp_path):
    exe = ROOT / "livespikesorter_gb300" / "lib" / "lss_replay"
    assert exe.exists()
    C, n = 64, 20_000
    rows = recording(n, C, seed=31)
    path = tmp_path / "rec.i16"
    rows.tofile(path)
    out = tmp_path / "out"
    r = subprocess.run([str(exe), "--tc", str(path), str(C), str(out), "3.5", "6000", "1500", "977"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = (out / "SpikeOutput_TC.txt").read_text().splitlines()
    means, medians = tc_oracle.calibrate(rows[:6000])
    ts, cs = [], []
    for s, m in replay_blocks(n, 977, 1500):
        t, c, _ = expect(rows[s:s + m], means, medians, 3.5, s)
        ts.append(t)
        cs.append(c)
    t = np.concatenate(ts)
    c = np.concatenate(cs)
    assert len(lines) == len(t) > 0
    assert lines[0] == f"{t[0]:20d},{c[0]:4d},0.000000"
    got = np.array([[int(a) for a in ln.split(",")[:2]] for ln in lines])
    np.testing.assert_array_equal(got[:, 0], t)
    np.testing.assert_array_equal(got[:, 1], c)
    assert r.stdout.strip() == f"events {len(t)}"


def test_gpu_reproduces_the_reference_run():
    """The events the reference's own ThresholdCrossing.cpp emitted on a scripted replay
    (tests/golden/tc_reference.npz, see tests/test_tc_reference_cpu.py): each fetched block pushed
    with the reference's stamp (its newest stream count) gives the same (time, channel) sequence."""
    import sys
    golden = ROOT / "tests" / "golden"
    sys.path.insert(0, str(golden))
    sys.path.insert(0, str(ROOT / "tests"))
    import make_tc_golden as mk
    from test_tc_reference_cpu import fetches
    z = np.load(golden / "tc_reference.npz")
    C = int(z["C"])
    x = mk.rows(z["means"], z["medians"], int(z["seed"]), int(z["N"]), C)
    times, chans = [], []
    with threshold.ThresholdCrossing(z["means"][:C], z["medians"][:C], float(z["threshold_std"]),
                                     max_rows=int(z["max_window"])) as tc:
        for latest, a, b in fetches(z):
            tc.push(np.ascontiguousarray(x[a:b]), first_row_sample=latest)
            ev = tc.poll_all()
            times.append(ev["time"])
            chans.append(ev["channel"])
    np.testing.assert_array_equal(np.concatenate(times), z["times"])
    np.testing.assert_array_equal(np.concatenate(chans), z["channels"])
