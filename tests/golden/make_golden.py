"""Generate the golden fixtures that pin the oracle to the reference's own code.

Runs only where the reference checkout is present (LSS_REFERENCE_DIR, else a "reference"
directory beside this repository); the fixtures it writes
(``*.npz`` beside this script) travel with the repository so the tests need no reference.

* ``kat_conv1d.npz``   -- the reference's known-answer script src/Python/conv1d_test.py,
                          executed unmodified with its file writes captured in memory.
* ``ks_window.npz``    -- one padded batch of a seeded 32-channel recording through the
                          vendored Kilosort 4.0.13 ``BinaryFiltered.filter`` (io.py:757-790),
                          ``prepare_matching`` / ``prepare_extract`` and ``run_matching``
                          (template_matching.py:20-26,110-202), all in float64.
* ``ks_stream.npz``    -- three batches (the last one partial) of the same recording through
                          the vendored ``extract`` (template_matching.py:28-85),
                          ``compute_spike_positions`` (postprocessing.py:33-46) and
                          ``remove_duplicates`` (postprocessing.py:9-30).

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import builtins
import contextlib
import importlib
import io
import os
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
REF = Path(os.environ.get("LSS_REFERENCE_DIR") or (REPO.parent / "reference"))
KS_DIR = REF / "src/Python/run_online_spikes/Lib/site-packages/kilosort"
sys.path.insert(0, str(REPO))


def load_kilosort():
    """Import the vendored Kilosort modules the hot path uses.  Siblings that need numba or
    faiss (absent here) are replaced by empty stubs; nothing on the matching path uses them."""
    def njit(*a, **k):
        if len(a) == 1 and callable(a[0]) and not k:
            return a[0]
        return lambda f: f
    numba = types.ModuleType("numba")
    numba.njit = njit
    ntypes = types.ModuleType("numba.types")
    ntypes.bool_ = np.bool_
    numba.types = ntypes
    sys.modules["numba"] = numba
    sys.modules["numba.types"] = ntypes
    pkg = types.ModuleType("kilosort")
    pkg.__path__ = [str(KS_DIR)]
    sys.modules["kilosort"] = pkg
    for name in ("spikedetect", "CCG", "clustering_qr"):
        stub = types.ModuleType("kilosort." + name)
        stub.xy_templates = None
        stub.get_data_cpu = None
        sys.modules["kilosort." + name] = stub
        setattr(pkg, name, stub)
    mods = {}
    for name in ("preprocessing", "template_matching", "postprocessing", "io"):
        mods[name] = importlib.import_module("kilosort." + name)
        setattr(pkg, name, mods[name])
    return mods


def run_conv1d_kat():
    """Execute src/Python/conv1d_test.py with ``open`` captured; return {name: values}."""
    captured = {}

    class _Sink(io.StringIO):
        def __init__(self, key):
            super().__init__()
            self.key = key

        def close(self):
            captured[self.key] = self.getvalue()
            super().close()

    def fake_open(path, mode="r", *a, **k):
        if "w" in mode:
            return _Sink(Path(str(path)).name)
        return builtins.open(path, mode, *a, **k)

    src = (REF / "src/Python/conv1d_test.py").read_text()
    ns = {"__name__": "conv1d_test", "open": fake_open}
    with contextlib.redirect_stdout(io.StringIO()):
        exec(compile(src, "conv1d_test.py", "exec"), ns)
    return {k: np.array([float(x) for x in v.split()]) for k, v in captured.items()}


def main():
    import torch
    from livespikesorter_gb300 import synth

    torch.set_default_dtype(torch.float64)
    ks = load_kilosort()

    # ---- known-answer test of the reference --------------------------------------------
    kat = run_conv1d_kat()
    np.savez_compressed(HERE / "kat_conv1d.npz", **{k: v for k, v in kat.items()})

    # ---- a seeded small recording and its export -----------------------------------------
    cfg = synth.SynthConfig(n_chan=32, n_units=12, n_samples=5500, rate_hz=25.0, drift_um=6.0,
                            whiten_batch=1500, whiten_batches=3, seed=7)
    rec = synth.make_recording(cfg)
    oss = synth.build_oss_input(rec)
    NT, nt, C = 2000, cfg.nt, cfg.n_chan
    d_last = float(synth.drift_um_at(cfg, cfg.n_samples - 1))
    xc64, yc64 = rec.xc.astype(np.float64), rec.yc.astype(np.float64)
    ops = {
        "settings": {"nearest_chans": cfg.n_nearest, "n_pcs": cfg.n_pcs, "sig_interp": 20.0},
        "nt": nt, "nt0min": cfg.nt0min, "Th_learned": cfg.th_learned, "batch_size": NT,
        "wPCA": torch.from_numpy(oss.wPCA.astype(np.float64)), "xc": xc64, "yc": yc64,
        "probe": {"xc": xc64, "yc": yc64}, "nblocks": 1, "yblk": np.zeros(1),
    }
    xp = np.stack([xc64, yc64], 1)
    Kxx = torch.from_numpy(synth.kernel2d(xp, xp, 20.0))
    ops["iKxx"] = torch.linalg.inv(Kxx + 0.01 * torch.eye(C))
    bfile = ks["io"].BinaryFiltered(
        None, C, fs=int(cfg.fs), NT=NT, nt=nt, nt0min=cfg.nt0min, chan_map=np.arange(C),
        hp_filter=torch.from_numpy(oss.hp_filter.astype(np.float64)),
        whiten_mat=torch.from_numpy(oss.whitening.astype(np.float64)),
        dshift=np.full(4, d_last), device=torch.device("cpu"), file_object=rec.data)
    U = torch.from_numpy(oss.Wall3.astype(np.float64))
    oss_arrays = dict(
        Wall3=oss.Wall3, wPCA=oss.wPCA, whitening=oss.whitening, drift=oss.drift,
        hp_filter=oss.hp_filter, xc=oss.xc, yc=oss.yc, centroids=oss.centroids,
        pre_wf=oss.pre_wf, ctc=oss.ctc, iCC=oss.iCC, iU=oss.iU, Ucc=oss.Ucc,
        misc=np.array([cfg.nt0min, cfg.n_nearest, cfg.th_learned, cfg.duplicate_spike_bins]))

    # ---- one window through the vendored filter + run_matching ----------------------------
    with contextlib.redirect_stdout(io.StringIO()):
        Xf = bfile.padded_batch_to_torch(1, ops)
        ctc = ks["template_matching"].prepare_matching(ops, U)
        iCC, iU, Ucc = ks["template_matching"].prepare_extract(ops, U, cfg.n_nearest, device="cpu")
        st, amps, Xres = ks["template_matching"].run_matching(ops, Xf.clone(), U, ctc, device="cpu")
    raw = rec.data[NT - nt: 2 * NT + nt]
    np.savez_compressed(
        HERE / "ks_window.npz", window=raw, X=Xf.numpy().astype(np.float32), st=st.numpy(), amps=amps.numpy()[:, 0],
        Xres=Xres.numpy().astype(np.float32), ctc_ks=ctc.numpy(), iCC_ks=iCC.numpy(), iU_ks=iU.numpy(), Ucc_ks=Ucc.numpy(),
        max_iters=np.array(100), NT=np.array(NT), **oss_arrays)

    # ---- the stream: extract + positions + duplicate removal -------------------------------
    with tempfile.TemporaryDirectory() as td, contextlib.redirect_stdout(io.StringIO()):
        stx, tF, ops2 = ks["template_matching"].extract(ops, Path(td), bfile, U, device=torch.device("cpu"))
        xs, ys = ks["postprocessing"].compute_spike_positions(torch.from_numpy(stx.astype(np.int64)), tF, ops2)
    times = stx[:, 0].astype(np.int64)
    d = (xs[:, None] - oss.centroids[None, :, 0]) ** 2 + (ys[:, None] - oss.centroids[None, :, 1]) ** 2
    clu = np.argmin(d, 1).astype(np.int32)
    _, _, keep = ks["postprocessing"].remove_duplicates(times, clu, cfg.duplicate_spike_bins)
    np.savez_compressed(
        HERE / "ks_stream.npz", data=rec.data, st=stx, tF=tF.numpy(), xs=np.asarray(xs), ys=np.asarray(ys),
        clu=clu, keep=np.asarray(keep), NT=np.array(NT), max_iters=np.array(100), **oss_arrays)
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
