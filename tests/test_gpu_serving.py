"""Several probe streams on one GPU at once (the reference runs one sorter thread per probe,
src/main.cpp:77-85; here one handle per stream, each on its own CUDA stream): handles of uneven
size driven concurrently from their own host threads with uneven pushes must give, bit for bit,
the spikes each stream gives when sorted alone."""
import threading

import numpy as np
import pytest

from livespikesorter_gb300 import sorter, synth

from lss_testutil import make_dataset

pytestmark = pytest.mark.gpu

STREAMS = [  # (channels, units, batch samples, seconds, seed)
    (96, 64, 1500, 1.0, 41),
    (64, 32, 750, 1.2, 42),
    (128, 96, 3000, 1.0, 43),
]


@pytest.fixture(scope="module")
def datasets(tmp_path_factory):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    out = []
    for C, T, NT, sec, seed in STREAMS:
        cfg = synth.SynthConfig(n_chan=C, n_units=T, n_samples=int(sec * 30000), seed=seed, rate_hz=15.0)
        d, data, _ = make_dataset(cfg, tmp_path_factory.mktemp(f"s{C}"))
        out.append((d, data, NT))
    return out


def _sort_alone(d, data, NT):
    with sorter.OnlineSorter(d, batch_samples=NT, max_iters=50) as s:
        return s.sort_stream(data, chunk=NT)


def _chunks(n, NT, seed):
    rng = np.random.default_rng(seed)
    sizes, s = [], 0
    while s < n:
        k = int(rng.integers(NT // 3, 2 * NT))
        sizes.append(min(k, n - s))
        s += sizes[-1]
    return sizes


def test_concurrent_streams_equal_alone(datasets):
    alone = [_sort_alone(d, data, NT) for d, data, NT in datasets]
    results = [None] * len(datasets)
    errors = []
    barrier = threading.Barrier(len(datasets))

    def run(i):
        d, data, NT = datasets[i]
        try:
            with sorter.OnlineSorter(d, batch_samples=NT, max_iters=50) as s:
                barrier.wait()
                got = []
                pos = 0
                for k in _chunks(data.shape[0], NT, seed=i):
                    s.push(data[pos:pos + k])
                    pos += k
                    got.append(s.poll())
                s.flush()
                got.append(s.poll_all())
                results[i] = np.concatenate(got)
        except Exception as e:   # surfaced below, after every thread finished
            errors.append(e)

    th = [threading.Thread(target=run, args=(i,)) for i in range(len(datasets))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    for ref, got in zip(alone, results):
        assert len(ref) > 50
        assert len(got) == len(ref)
        for f in ("time", "tmpl", "cluster", "amp", "x", "y", "pcfeat"):
            np.testing.assert_array_equal(got[f], ref[f], err_msg=f)


def test_pinned_and_pageable_pushes_agree(datasets):
    """Page-locked rows go straight to the device (lss_push_batch returns once they are there, so
    the caller may reuse the buffer at once); pageable rows go through the pinned staging.  Uneven
    pushes alternating between the two -- the page-locked buffer overwritten right after each push
    -- give the spikes of the pageable stream, bit for bit."""
    torch = pytest.importorskip("torch")
    d, data, NT = datasets[0]
    ref = _sort_alone(d, data, NT)
    buf = torch.empty((3 * NT, data.shape[1]), dtype=torch.int16).pin_memory().numpy()
    rng = np.random.default_rng(7)
    got = []
    with sorter.OnlineSorter(d, batch_samples=NT, max_iters=50, group_batches=2) as s:
        pos, i = 0, 0
        while pos < data.shape[0]:
            k = min(int(rng.integers(NT // 4, 3 * NT)), data.shape[0] - pos)
            if i % 2 == 0:
                buf[:k] = data[pos:pos + k]
                s.push(buf[:k])
                buf[:k] = -12345
            else:
                s.push(data[pos:pos + k])
            pos += k
            i += 1
            got.append(s.poll())
        s.flush()
        got.append(s.poll_all())
    got = np.concatenate(got)
    assert len(got) == len(ref) > 50
    for f in ("time", "tmpl", "cluster", "amp", "x", "y", "pcfeat"):
        np.testing.assert_array_equal(got[f], ref[f], err_msg=f)
