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


def test_pc_score_cluster_rule_restated():
    """The oracle's PC-score rule against a line-by-line transcription of
    OnlineKilosort.py:233-284 (scores 2 X mu^T - |mu|^2, clusters beyond R masked to -inf, torch
    argmax = first maximum, -1 when no cluster is within R), on features with exact ties, spikes
    with no cluster in range and a NaN position."""
    rng = np.random.default_rng(5)
    N, nC, K, Tf, R = 200, 4, 3, 12, 30.0
    tF = rng.integers(-3, 4, (N, nC, K)).astype(np.float64)
    mu = rng.integers(-2, 3, (Tf, nC * K)).astype(np.float64)
    mu[7] = mu[2]                                  # duplicate centroid features: exact score ties
    cent = rng.uniform(0, 100, (Tf, 2))
    cent[7] = cent[2]
    xs, ys = rng.uniform(-20, 120, N), rng.uniform(-20, 120, N)
    xs[0] = np.nan
    got = ko.pc_score_cluster(tF, xs, ys, cent, mu, R)
    want = []
    for i in range(N):
        X = tF[i].reshape(-1)
        best, bs, any_in = 0, -np.inf, False
        for k in range(Tf):
            d2 = (xs[i] - cent[k, 0]) ** 2 + (ys[i] - cent[k, 1]) ** 2
            s = 2 * X @ mu[k] - (mu[k] ** 2).sum() if d2 <= R * R else -np.inf
            any_in |= bool(d2 <= R * R)
            if s > bs:
                best, bs = k, s
        want.append(best if any_in else -1)
    np.testing.assert_array_equal(got, np.array(want))
    assert got[0] == -1 and (got == -1).sum() > 5 and (got >= 0).sum() > 50
    assert not np.any(got == 7)                    # the tie always resolves to the first cluster
