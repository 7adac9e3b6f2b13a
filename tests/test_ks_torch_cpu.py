"""The torch (float32, CPU) form of the oracle that times the CPU baseline runs Kilosort's path
like the numpy oracle: on the vendored-Kilosort golden window and on a seeded 96-channel window it
finds the same spikes (>= 99.5 %, amplitudes within 1e-3 relative) with the same preprocessing
(within 1e-4 of the largest magnitude)."""
import numpy as np
import pytest

from livespikesorter_gb300 import synth
from oracle import ks_oracle as ko

from lss_testutil import agreement, make_dataset

torch = pytest.importorskip("torch")


def _check(window_CW, oss, max_iters):
    from oracle import ks_torch
    ref = ko.sort_window(window_CW, oss, max_iters=max_iters)
    X = ks_torch.preprocess(window_CW, oss)
    np.testing.assert_allclose(X.numpy(), ref.X, rtol=0, atol=1e-4 * np.abs(ref.X).max())
    st, amps, _, tF, xs, ys = ks_torch.Matcher(oss).run(X, max_iters=max_iters)
    st = st.numpy()
    a, amp_ok, amax = agreement(ref.match.st[:, 0], ref.match.st[:, 1], ref.match.amps, st[:, 0], st[:, 1],
                                amps.numpy())
    assert len(ref.match.st) > 10
    assert a >= 0.995 and amp_ok >= 0.995, (a, amp_ok, amax)


def test_golden_window(golden_dir):
    z = np.load(golden_dir / "ks_window.npz")
    _check(z["window"].T, ko.oss_from_arrays(z), int(z["max_iters"]))


def test_seeded_96ch(tmp_path):
    cfg = synth.SynthConfig(n_chan=96, n_units=64, n_samples=6000 + 122, seed=4, whiten_batch=2000,
                            whiten_batches=3)
    d, data, _ = make_dataset(cfg, tmp_path)
    _check(data[: 6000 + 122].T, ko.load_oss_input(d), 50)
