"""Pin the oracle to the reference: the reference's own known-answer script
(src/Python/conv1d_test.py) and the vendored Kilosort 4.0.13 code run on seeded inputs
(fixtures written by tests/golden/make_golden.py)."""
import numpy as np
import pytest

from oracle import ks_oracle as ko


@pytest.fixture(scope="module")
def kat(golden_dir):
    return np.load(golden_dir / "kat_conv1d.npz")


@pytest.fixture(scope="module")
def win(golden_dir):
    return np.load(golden_dir / "ks_window.npz")


@pytest.fixture(scope="module")
def stream(golden_dir):
    return np.load(golden_dir / "ks_stream.npz")


def test_kat_conv1d(kat):
    """Every intermediate of conv1d_test.py: basis conv, projection, Cf, per-sample max, pool."""
    X = kat["batch"].reshape(2, 11)
    W = kat["wPCA"].reshape(3, 3)
    U = kat["Wall3"].reshape(2, 3, 2)
    nm = 1.0 / kat["nm"]                      # the script writes reciprocal(nm)
    np.testing.assert_allclose(nm, [42, 45])
    np.testing.assert_array_equal(ko.conv_basis(X, W).ravel(), kat["batchPCA"])
    B = ko.project(X, U, W)
    np.testing.assert_array_equal(B.ravel(), kat["convResult"])
    Cf, Cfmax, imax, Cmax = ko.scores(B, nm, 3)
    np.testing.assert_allclose(Cf.ravel(), kat["Cf"], rtol=1e-12)
    np.testing.assert_allclose(Cfmax, kat["Cfmax"], rtol=1e-12)
    np.testing.assert_allclose(Cmax, kat["Cmax"], rtol=1e-12)
    ctc = kat["ctc_permuted"].reshape(1, 2, 3)
    np.testing.assert_array_equal(ctc[kat["spike_templates"].astype(int)].ravel(), kat["ctc_sub"])


def test_preprocess_matches_kilosort_filter(win):
    oss = ko.oss_from_arrays(win)
    X = ko.preprocess(win["window"].T, oss)
    ref = win["X"].astype(np.float64)
    assert X.shape == ref.shape
    scale = np.abs(ref).max()
    np.testing.assert_allclose(X, ref, atol=2e-6 * scale, rtol=0)


def test_exporter_matches_kilosort_prepare(win):
    """The exporter's ctc / iCC / iU / Ucc equal Kilosort's prepare_matching / prepare_extract."""
    from livespikesorter_gb300 import synth
    ctc = synth.prepare_matching(win["wPCA"], win["Wall3"])
    np.testing.assert_allclose(ctc, win["ctc_ks"], rtol=1e-5, atol=1e-6 * np.abs(win["ctc_ks"]).max())
    iCC, iU, Ucc = synth.prepare_extract(win["xc"].astype(np.float64), win["yc"].astype(np.float64),
                                         win["Wall3"], int(win["misc"][1]))
    np.testing.assert_array_equal(iU, win["iU_ks"])
    np.testing.assert_allclose(Ucc, win["Ucc_ks"], rtol=1e-6)
    np.testing.assert_array_equal(iCC, win["iCC_ks"])


def test_run_matching_matches_kilosort(win):
    oss = ko.oss_from_arrays(win)
    X = win["X"].astype(np.float64)
    m = ko.run_matching(X, win["Wall3"], win["wPCA"], win["ctc_ks"], oss.th_learned,
                        max_iters=int(win["max_iters"]), amp_dtype=np.float32)
    np.testing.assert_array_equal(m.st, win["st"])
    np.testing.assert_allclose(m.amps, win["amps"], rtol=1e-5)
    np.testing.assert_allclose(m.Xres, win["Xres"], atol=1e-5 * np.abs(win["Xres"]).max())
    assert len(m.st) > 5


def test_sort_stream_matches_kilosort_extract(stream):
    oss = ko.oss_from_arrays(stream)
    res = ko.sort_stream(stream["data"], oss, int(stream["NT"]), max_iters=int(stream["max_iters"]))
    st = stream["st"]
    order = np.lexsort((st[:, 1], st[:, 0]))
    st = st[order]
    np.testing.assert_array_equal(res["time"], st[:, 0].astype(np.int64))
    np.testing.assert_array_equal(res["template"], st[:, 1].astype(np.int64))
    np.testing.assert_allclose(res["amp"], st[:, 2], rtol=2e-5)
    np.testing.assert_allclose(res["tF"], stream["tF"][order], atol=1e-4 * np.abs(stream["tF"]).max())
    np.testing.assert_allclose(res["x"], stream["xs"][order], atol=1e-3)
    np.testing.assert_allclose(res["y"], stream["ys"][order], atol=1e-3)
    np.testing.assert_array_equal(res["cluster"], stream["clu"][order])
    np.testing.assert_array_equal(res["keep"], stream["keep"][order])


def test_cnpy_semantics_ignore_fortran_order(tmp_path):
    """drift_matrix.npy is written Fortran-ordered (``M.T``); cnpy-style reading yields M."""
    M = np.arange(12, dtype=np.float32).reshape(3, 4)
    np.save(tmp_path / "m.npy", M.T)
    assert np.load(tmp_path / "m.npy").flags.f_contiguous
    got = ko.read_npy_cnpy(tmp_path / "m.npy")
    assert got.shape == (4, 3)
    np.testing.assert_array_equal(got.ravel(), M.ravel())
