"""Template subsetting of an oss_input/ directory (lss_subset_plan / lss_subset_write, in place of
the reference's subset_templates.py) without a GPU: the n most active preclustered templates by
spike count (ties by energy), or by energy; the channel-range filter on each template's Wall3
energy per channel, composed before the cap; every preclustered axis cut consistently (ctc on
both), final-cluster and channel files untouched byte for byte, the manifest, the error cases --
and the result loads through the library's own loader (which then stops at the missing GPU, not at
a shape check)."""
import ctypes as ct
import json

import numpy as np
import pytest

from livespikesorter_gb300 import sorter, subset, synth


@pytest.fixture(scope="module")
def oss_dir(tmp_path_factory):
    cfg = synth.SynthConfig(n_chan=32, n_units=12, n_samples=6000, rate_hz=20.0, whiten_batch=2000,
                            whiten_batches=2, seed=8)
    rec = synth.make_recording(cfg)
    d = tmp_path_factory.mktemp("sub") / "oss_input"
    synth.write_oss_input(synth.build_oss_input(rec), d)
    return d


def _load_status(d):
    lib = sorter.load_library()
    p = sorter.default_params()
    h = ct.c_void_p()
    st = lib.lss_open(str(d).encode(), ct.byref(p), ct.byref(h))
    if st == 0:
        lib.lss_close(h)
    return st, (lib.lss_last_error(None) or b"").decode()


def test_most_active_templates_kept(oss_dir, tmp_path):
    out = tmp_path / "o"
    m = subset.subset_oss_input(oss_dir, out, n=5)
    keep = np.array(m["kept_indices"])
    assert m["metric"] == "spike count" and m["new_unclu_T"] == 5 and list(keep) == sorted(keep)
    counts = np.bincount(np.load(oss_dir / "spike_detection_templates.npy"), minlength=12)
    dropped = np.setdiff1d(np.arange(12), keep)
    assert counts[keep].min() >= counts[dropped].max()
    W = np.load(oss_dir / "Wall3.npy")
    np.testing.assert_array_equal(np.load(out / "Wall3.npy"), W[keep])
    ctc = np.load(oss_dir / "ctc.npy")
    np.testing.assert_array_equal(np.load(out / "ctc.npy"), ctc[keep][:, keep])
    np.testing.assert_array_equal(np.load(out / "Ucc.npy"), np.load(oss_dir / "Ucc.npy")[:, keep])
    np.testing.assert_array_equal(np.load(out / "iU.npy"), np.load(oss_dir / "iU.npy")[keep])
    np.testing.assert_array_equal(np.load(out / "preclustered_template_waveforms.npy"),
                                  np.load(oss_dir / "preclustered_template_waveforms.npy")[keep])
    for f in ("templates.npy", "cluster_centroids.npy", "iCC.npy", "whiteningMat.npy", "wPCA.npy", "drift_matrix.npy"):
        assert (out / f).read_bytes() == (oss_dir / f).read_bytes()
    assert (out / "misc.txt").read_text() == (oss_dir / "misc.txt").read_text()
    assert json.loads((out / "subset_manifest.json").read_text())["kept_indices"] == list(keep)
    st, msg = _load_status(out)
    assert st == 4, msg      # loaded and validated; no GPU here


def _energy(d):
    W = np.load(d / "Wall3.npy").astype(np.float64)
    return (W ** 2).sum(1)                                # [unclu_T, C]


def test_energy_metric_and_channel_range(oss_dir, tmp_path):
    m = subset.subset_oss_input(oss_dir, tmp_path / "n", n=4, metric="energy")
    e = _energy(oss_dir).sum(1)
    keep = np.array(m["kept_indices"])
    assert m["metric"] == "template energy" and e[keep].min() >= np.delete(e, keep).max()
    # channel range first, then the cap: templates whose strongest channel is in 0..15
    peak = _energy(oss_dir).argmax(1)
    on = np.where(peak <= 15)[0]
    assert 0 < len(on) < 12
    m2 = subset.subset_oss_input(oss_dir, tmp_path / "c", n=0, channel_range=(0, 15))
    assert m2["kept_indices"] == list(on) and m2["channel_filter"]["probe_channels_in_range"] == 16
    if len(on) > 2:
        m3 = subset.subset_oss_input(oss_dir, tmp_path / "c2", n=2, channel_range=(0, 15))
        assert set(m3["kept_indices"]) <= set(on) and len(m3["kept_indices"]) == 2
    # overlap: any in-range channel with RMS >= 0.1 of the strongest's
    en = _energy(oss_dir)
    ov = np.where(((en >= 0.01 * en.max(1, keepdims=True)) & (np.arange(en.shape[1]) <= 15)[None]).any(1))[0]
    assert set(on) <= set(ov)
    if len(ov) < 12:
        m4 = subset.subset_oss_input(oss_dir, tmp_path / "ov", channel_range=(0, 15), channel_criterion="overlap")
        assert m4["kept_indices"] == list(ov)
    else:
        with pytest.raises(subset.SubsetError):   # every template reaches the range: nothing to cut
            subset.subset_oss_input(oss_dir, tmp_path / "ov", channel_range=(0, 15), channel_criterion="overlap")
    assert subset.plan(oss_dir, subset.make_spec(channel_range=(0, 15), channel_criterion="overlap")) == list(ov)
    assert subset.main([str(oss_dir), str(tmp_path / "cli"), "--n-templates", "3"]) == 0
    assert json.loads((tmp_path / "cli" / "subset_manifest.json").read_text())["new_unclu_T"] == 3


def test_errors_and_inplace(oss_dir, tmp_path):
    with pytest.raises(subset.SubsetError):
        subset.subset_oss_input(oss_dir, tmp_path / "x", n=0)              # keeps everything
    (tmp_path / "exists").mkdir()
    with pytest.raises(subset.SubsetError):
        subset.subset_oss_input(oss_dir, tmp_path / "exists", n=3)
    with pytest.raises(subset.SubsetError):
        subset.subset_oss_input(oss_dir, tmp_path / "y", n=3, channel_range=(900, 999))
    import shutil
    d = tmp_path / "inplace"
    shutil.copytree(oss_dir, d)
    r = subset.subset_oss_input_inplace(d, n=7)
    assert r["applied"] and np.load(d / "Wall3.npy").shape[0] == 7 and np.load(d / "ctc.npy").shape[:2] == (7, 7)
    assert subset.subset_oss_input_inplace(d, n=0)["applied"] is False
    assert _load_status(d)[0] == 4
