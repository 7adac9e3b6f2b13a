"""Time the reference's own Kilosort CPU path on the bench workload -- MEASUREMENT RECIPE, run by
hand where the reference checkout is.

The per-batch path the GPU sorter replaces, as the reference runs it in Python: the vendored
Kilosort 4.0.13 (src/Python/run_online_spikes/Lib/site-packages/kilosort) ``BinaryFiltered``
preprocessing of a padded batch (io.py:757-790) and ``run_matching`` (template_matching.py:128-202),
float32 torch on the host's cores (torch.set_num_threads(os.cpu_count())), stdout silenced (the
vendored copy prints debug lines every call).  The workload is the bench's: 384 channels, 500
templates, 1500-sample batches + 2 x 61 context, 50 iterations.  The reference's Python cannot
travel to the GPU host, so this runs here; the numpy port (bench.py's reference arm) is timed on
the same batches beside it for scale.

    python oracle/time_vendored.py [n_batches]
"""
from __future__ import annotations

import contextlib
import io
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tests" / "golden"))


def main(n_batches: int = 6):
    import torch
    from make_golden import load_kilosort   # the vendored modules, numba / faiss stubbed
    from livespikesorter_gb300 import synth
    from oracle import ks_oracle as ko
    torch.set_num_threads(os.cpu_count())
    ks = load_kilosort()
    cfg = synth.SynthConfig(n_chan=384, n_units=500, n_samples=(n_batches + 3) * 1500 + 300, drift_um=20.0,
                            whiten_batch=3000, whiten_batches=3, seed=1)
    rec = synth.make_recording(cfg)
    oss = synth.build_oss_input(rec)
    NT, nt, C = 1500, cfg.nt, cfg.n_chan
    d_last = float(synth.drift_um_at(cfg, cfg.n_samples - 1))
    xc, yc = rec.xc.astype(np.float32), rec.yc.astype(np.float32)   # float32 probe: the drift matrix in float32
    ops = {"settings": {"nearest_chans": cfg.n_nearest, "n_pcs": cfg.n_pcs, "sig_interp": 20.0},
           "nt": nt, "nt0min": cfg.nt0min, "Th_learned": cfg.th_learned, "batch_size": NT,
           "wPCA": torch.from_numpy(oss.wPCA.astype(np.float32)), "xc": xc, "yc": yc,
           "probe": {"xc": xc, "yc": yc}, "nblocks": 1, "yblk": np.zeros(1)}
    xp = np.stack([xc, yc], 1)
    Kxx = torch.from_numpy(synth.kernel2d(xp, xp, 20.0).astype(np.float32))
    ops["iKxx"] = torch.linalg.inv(Kxx + 0.01 * torch.eye(C))
    bfile = ks["io"].BinaryFiltered(None, C, fs=int(cfg.fs), NT=NT, nt=nt, nt0min=cfg.nt0min, chan_map=np.arange(C),
                                    hp_filter=torch.from_numpy(oss.hp_filter.astype(np.float32)),
                                    whiten_mat=torch.from_numpy(oss.whitening.astype(np.float32)),
                                    dshift=np.full(n_batches + 4, d_last), device=torch.device("cpu"),
                                    file_object=rec.data)
    U = torch.from_numpy(oss.Wall3.astype(np.float32))
    with contextlib.redirect_stdout(io.StringIO()):
        ctc = ks["template_matching"].prepare_matching(ops, U)
        times = []
        for j in range(1, n_batches + 2):
            t0 = time.perf_counter()
            X = bfile.padded_batch_to_torch(j, ops)
            ks["template_matching"].run_matching(ops, X, U, ctc, device="cpu")
            times.append(time.perf_counter() - t0)
    times = times[1:]   # the first batch warms up
    rate = NT * C / float(np.median(times))
    print(f"vendored Kilosort (filter + run_matching), torch {torch.__version__} float32 on {os.cpu_count()} "
          f"threads: median {1e3 * np.median(times):.1f} ms per 1500-sample batch = {rate / 1e6:.2f} M ch*samples/s")
    # the numpy port on the same batches
    o = ko.load_oss_input(synth.write_oss_input(oss, Path(os.environ.get("TMPDIR", "/tmp")) / "tv_oss"))
    tp = []
    for j in range(1, n_batches + 1):
        t0 = time.perf_counter()
        ko.sort_window(ko.padded_batch(rec.data, j, NT, nt), o, max_iters=50, dtype=np.float32)
        tp.append(time.perf_counter() - t0)
    print(f"numpy port (float32): median {1e3 * np.median(tp):.1f} ms per batch = "
          f"{NT * C / float(np.median(tp)) / 1e6:.2f} M ch*samples/s")
    # the torch form of the port (bench.py's CPU baseline and reference arm)
    from oracle import ks_torch
    mt = ks_torch.Matcher(o)
    tt = []
    for j in range(0, n_batches + 1):
        t0 = time.perf_counter()
        X = ks_torch.preprocess(ko.padded_batch(rec.data, 1 + j % n_batches, NT, nt), o)
        mt.run(X, max_iters=50)
        tt.append(time.perf_counter() - t0)
    tt = tt[1:]
    print(f"torch port (float32, {torch.get_num_threads()} threads): median {1e3 * np.median(tt):.1f} ms per batch = "
          f"{NT * C / float(np.median(tt)) / 1e6:.2f} M ch*samples/s")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 6)
