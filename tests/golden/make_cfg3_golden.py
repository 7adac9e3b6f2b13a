"""Generate tests/golden/cfg3_full_oracle.npz: the float64 oracle (oracle/ks_oracle.py, Kilosort's
preprocessing and matching loop) on the full dense shape -- 384 channels, 1000 templates, one
60000-sample batch, 30 Hz with 30 % of spikes overlapping within 1 ms -- a run of several minutes
on a CPU, kept as a fixture: the spikes (time, template, amplitude) and a digest of the seeded
input the test regenerates (livespikesorter_gb300.synth, the same config).

    python tests/golden/make_cfg3_golden.py
"""
from __future__ import annotations

import hashlib
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]


def config():
    sys.path.insert(0, str(ROOT))
    from livespikesorter_gb300 import synth
    return synth.SynthConfig(n_chan=384, n_units=1000, n_samples=60000 + 122, rate_hz=30.0, overlap_frac=0.3,
                             whiten_batch=6000, whiten_batches=3, seed=23)


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    from lss_testutil import make_dataset
    from oracle import ks_oracle as ko
    t0 = time.time()
    with tempfile.TemporaryDirectory() as td:
        d, data, _ = make_dataset(config(), td)
        oss = ko.load_oss_input(d)
        win = data[: 60000 + 122]
        r = ko.sort_window(win.T, oss, max_iters=50)
        wall3 = np.load(Path(d) / "Wall3.npy")
    nt, nt0 = oss.wPCA.shape[1], oss.nt0min
    np.savez_compressed(HERE / "cfg3_full_oracle.npz", time=(r.match.st[:, 0] - nt // 2 + nt0).astype(np.int64),
                        template=r.match.st[:, 1].astype(np.int32), amp=r.match.amps.astype(np.float64),
                        data_sha256=digest(win), wall3_sha256=digest(wall3), max_iters=50)
    print(f"{len(r.match.st)} spikes in {time.time() - t0:.0f} s -> {HERE / 'cfg3_full_oracle.npz'}")


if __name__ == "__main__":
    main()
