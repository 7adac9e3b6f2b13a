"""The acquisition loop's behind/skip policy (OnlineSpikesV2.cu:705-746) on the host: the C++ loop
of lss::OnlineSpikesV2 (lss::run_ingest_loop, include/lss_online_spikes_v2.hpp) is compiled with g++
against a scripted DataSocket and each of the reference's five branches is checked by the start
sample of the fetch it makes and the skip count.

Reference branches, with latest = the stream sample count after the wait, processed = one past the
last row handed to the sorter, allowedCt = latest - iTimeBehind ms of samples:
  latest - processed <= maxWindow        -> rows from processed               (no skip)
  else iTimeBehind == 0                  -> the newest maxWindow rows          (skip)
  else processed >= allowedCt            -> rows from processed (catch up)     (no skip)
  else bSmallskip                        -> rows from allowedCt                (skip)
  else                                   -> the newest maxWindow rows          (skip)
"""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    exe = tmp_path_factory.mktemp("ingest") / "ingest_policy_driver"
    subprocess.run([gxx, "-O1", "-std=c++17", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "ingest_policy_driver.cpp"), "-o", str(exe)], check=True)
    return exe


def run(driver, script, first=0, max_rows=1500, min_rows=82, behind_ms=0, rate=30000.0, small=False):
    inp = f"{max_rows} {min_rows} {behind_ms} {rate} {int(small)} {first} {len(script)} " + " ".join(map(str, script))
    out = subprocess.run([str(driver)], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    pushes = [tuple(int(v) for v in ln.split()) for ln in out if ln and not ln.startswith("skips")]
    skips = int([ln for ln in out if ln.startswith("skips")][0].split()[1])
    return pushes, skips


def test_normal_fetches_continue_from_processed(driver):
    # 1000 new rows per wait: never more than one batch behind
    pushes, skips = run(driver, [1000, 2000, 3000], first=0)
    assert [(p[0], p[1]) for p in pushes] == [(0, 1000), (1000, 1000), (2000, 1000)]
    assert skips == 0
    # rows carry their own stream sample: the fetch delivered the rows it names
    assert all(p[2] == p[0] and p[3] == p[0] + p[1] - 1 for p in pushes)


def test_no_lag_allowed_jumps_to_newest_batch(driver):
    # iTimeBehind = 0: 4000 rows behind after the second wait -> the newest 1500 (2500..3999)
    pushes, skips = run(driver, [1000, 5000, 6000], first=0, behind_ms=0)
    assert [(p[0], p[1]) for p in pushes] == [(0, 1000), (3500, 1500), (5000, 1000)]
    assert skips == 1


def test_catch_up_within_allowed_lag(driver):
    # 100 ms allowed = 3000 samples; 2500 behind (> one batch, < allowed): from processed, no skip
    pushes, skips = run(driver, [1000, 3500, 3600], first=0, behind_ms=100)
    assert [(p[0], p[1]) for p in pushes] == [(0, 1000), (1000, 1500), (2500, 1100)]
    assert skips == 0


def test_small_skip_starts_at_allowed_count(driver):
    # 10 ms allowed = 300 samples; 9000 behind: allowedCt = 10000 - 300 = 9700
    pushes, skips = run(driver, [1000, 10000, 11000], first=0, behind_ms=10, small=True)
    assert [(p[0], p[1]) for p in pushes] == [(0, 1000), (9700, 300), (10000, 1000)]
    assert skips == 1


def test_big_skip_takes_newest_batch(driver):
    # the same lag without small skip: the newest 1500 rows (8500..9999)
    pushes, skips = run(driver, [1000, 10000, 11000], first=0, behind_ms=10, small=False)
    assert [(p[0], p[1]) for p in pushes] == [(0, 1000), (8500, 1500), (10000, 1000)]
    assert skips == 1


def test_lag_grows_without_bound_only_when_allowed(driver):
    # a source 2x faster than one batch per wait: with a large allowance the loop keeps catching up
    # from processed (never skips); without it every behind step jumps
    script = [3000 * k for k in range(1, 8)]
    pushes, skips = run(driver, script, first=0, behind_ms=100000)
    assert skips == 0 and pushes[0][0] == 0
    assert all(b[0] == a[0] + a[1] for a, b in zip(pushes, pushes[1:]))
    pushes, skips = run(driver, script, first=0, behind_ms=0)
    assert skips == len(script)
    assert all(p[0] + p[1] == s for p, s in zip(pushes, script))
