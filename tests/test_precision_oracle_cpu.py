"""The precision-study oracle (oracle/precision_oracle.py): its exact variants are Kilosort's loop
(ks_oracle.run_matching) on the golden window, its rounding matches the formats' grids, and
re-scoring makes the amplitudes of the spikes it keeps exact."""
import numpy as np
import pytest

from oracle import ks_oracle as ko
from oracle import precision_oracle as po


@pytest.fixture(scope="module")
def window(golden_dir):
    z = np.load(golden_dir / "ks_window.npz")
    oss = ko.oss_from_arrays(z)
    X = ko.preprocess(z["window"].T, oss)
    return X, oss, int(z["max_iters"])


def test_exact_variants_are_kilosorts_loop(window):
    X, oss, it = window
    ref = ko.run_matching(X, oss.Wall3, oss.wPCA, oss.ctc, oss.th_learned, max_iters=it)
    for kw in ({}, {"keep": oss.Wall3.shape[0]}, {"rescore": True}):
        st, amps = po.run_matching_variant(X, oss.Wall3, oss.wPCA, oss.ctc, oss.th_learned, max_iters=it, **kw)
        np.testing.assert_array_equal(st, ref.st)
        np.testing.assert_allclose(amps, ref.amps, rtol=1e-12)


def test_rounding_grids():
    assert po.round_fp8(448.0, "e4m3") == 448.0 and po.round_fp8(1e6, "e4m3") == 448.0
    assert po.round_fp8(1.0625, "e4m3") == 1.0          # 1 + 1/16 ties to the even neighbour
    assert po.round_fp8(1.1875, "e4m3") == 1.25
    assert po.round_fp8(2.0 ** -9, "e4m3") == 2.0 ** -9  # smallest subnormal
    assert po.round_fp8(-3.0, "e5m2") == -3.0 and po.round_fp8(3.25, "e5m2") == 3.0
    assert po.round_bf16(np.float32(1.00390625)) == 1.0  # 1 + 2^-8 ties to even
    x = np.random.default_rng(0).normal(0, 10, 1000)
    assert np.max(np.abs(po.round_fp8(x, "e4m3") - x) / np.maximum(np.abs(x), 2.0 ** -6)) <= 2.0 ** -4 + 1e-12


def test_rescored_amplitudes_are_exact_for_the_spikes_kept(window):
    X, oss, it = window
    ref = ko.run_matching(X, oss.Wall3, oss.wPCA, oss.ctc, oss.th_learned, max_iters=it)
    st, amps = po.run_matching_variant(X, oss.Wall3, oss.wPCA, oss.ctc, oss.th_learned, fmt="e4m3", rescore=True,
                                       max_iters=it)
    # where the accepted sequence matches Kilosort's (spike for spike, in order), so does every amplitude
    n = 0
    while n < min(len(st), len(ref.st)) and tuple(st[n]) == tuple(ref.st[n]):
        n += 1
    assert n > 0
    np.testing.assert_allclose(amps[:n], ref.amps[:n], rtol=1e-9)


def test_static_scales_fold_into_the_templates_and_saturate(window):
    """The static-scale projection (the FP8 kernel's form): scales calibrated on the window itself
    stay within e4m3's relative error of the exact product, and a held-out value beyond twice the
    calibrated range saturates at the largest finite value times its scale."""
    X, oss, _ = window
    U2, Bpc2 = po.operands(X, oss.Wall3, oss.wPCA)
    s = po.calibrate_act_scale(Bpc2)
    assert s.shape == (Bpc2.shape[0], 1) and np.all(s > 0)
    np.testing.assert_allclose(s[:, 0], 2 * np.abs(Bpc2).max(1) / 448.0)
    Bq = po.project_rounded(U2, Bpc2, "e4m3", act_scale=s)
    Be = U2 @ Bpc2
    # each product term carries at most (1 + 2^-4)^2 - 1 relative error, plus subnormal flushes
    bound = (np.abs(U2) @ np.abs(Bpc2)) * ((1 + 2.0 ** -4) ** 2 - 1) + 1e-6 * np.abs(Be).max()
    assert np.all(np.abs(Bq - Be) <= bound)
    big = Bpc2.copy()
    big[0, 0] = 10 * np.abs(Bpc2[0]).max()
    e = np.zeros((1, U2.shape[1]))
    e[0, 0] = 1.0
    assert po.project_rounded(e, big[:, :1], "e4m3", act_scale=s)[0, 0] == pytest.approx(448.0 * s[0, 0], rel=2 ** -3)


def test_static_rescored_variant_keeps_exact_amplitudes(window):
    X, oss, it = window
    ref = ko.run_matching(X, oss.Wall3, oss.wPCA, oss.ctc, oss.th_learned, max_iters=it)
    s = po.calibrate_act_scale(po.operands(X, oss.Wall3, oss.wPCA)[1])
    st, amps = po.run_matching_variant(X, oss.Wall3, oss.wPCA, oss.ctc, oss.th_learned, fmt="e4m3", rescore=True,
                                       max_iters=it, act_scale=s)
    n = 0
    while n < min(len(st), len(ref.st)) and tuple(st[n]) == tuple(ref.st[n]):
        n += 1
    assert n > 0
    np.testing.assert_allclose(amps[:n], ref.amps[:n], rtol=1e-9)


def test_widened_lists_between_the_fixed_lengths(window):
    """Widened lists (keep_wide at crowded samples): with no sample crowded they are the keep-entry
    lists, with every sample crowded the keep_wide-entry ones."""
    X, oss, it = window
    T = oss.Wall3.shape[0]
    k, kw = 4, 8
    assert T > kw
    args = (X, oss.Wall3, oss.wPCA, oss.ctc, oss.th_learned)
    fixed_k = po.run_matching_variant(*args, keep=k, max_iters=it)
    fixed_kw = po.run_matching_variant(*args, keep=kw, max_iters=it)
    none = po.run_matching_variant(*args, keep=k, keep_wide=kw, crowd=np.inf, max_iters=it)
    every = po.run_matching_variant(*args, keep=k, keep_wide=kw, crowd=-1.0, max_iters=it)
    np.testing.assert_array_equal(none[0], fixed_k[0])
    np.testing.assert_array_equal(none[1], fixed_k[1])
    np.testing.assert_array_equal(every[0], fixed_kw[0])
    np.testing.assert_array_equal(every[1], fixed_kw[1])
