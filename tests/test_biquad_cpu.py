"""The stateful high-pass mode without a GPU: the library's Butterworth sections against
scipy.signal.butter (Kilosort's design, KS/preprocessing.py:121-136), the float64 oracle's
chunked filtering, a float64 restatement of the kernels' three-pass chunked recurrence (zero-state
chunk ends, scan with the chunk transition matrix, re-run from the entering state) against
scipy.signal.sosfilt, the oracle's stream framing, and the parameter checks of lss_open."""
import ctypes as ct

import numpy as np
import pytest

from livespikesorter_gb300 import sorter, synth
from oracle import ks_oracle as ko

signal = pytest.importorskip("scipy.signal")


@pytest.mark.parametrize("order,fc", [(1, 300.0), (2, 150.0), (3, 300.0), (3, 1000.0), (4, 300.0)])
def test_sections_match_scipy(order, fc):
    got = sorter.butter_highpass_sos(order, fc, 30000.0)
    ref = signal.butter(order, fc, btype="high", fs=30000.0, output="sos")
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13)


def test_sections_reject_bad_arguments():
    for args in ((0, 300.0, 30000.0), (5, 300.0, 30000.0), (3, 15000.0, 30000.0), (3, -1.0, 30000.0)):
        with pytest.raises(sorter.SorterError):
            sorter.butter_highpass_sos(*args)


def _cascade(sos, x, z):
    """Direct form II transposed, float64, state z [n_sections, 2] updated in place."""
    y = np.empty_like(x)
    for n, v in enumerate(x):
        u = v
        for s, (b0, b1, b2, _, a1, a2) in enumerate(sos):
            o = b0 * u + z[s, 0]
            z[s, 0] = b1 * u - a1 * o + z[s, 1]
            z[s, 1] = b2 * u - a2 * o
            u = o
        y[n] = u
    return y


def test_chunked_recurrence_equals_sosfilt():
    """The kernels' method in float64: zero-state chunk ends, the entering states by
    s[k+1] = P s[k] + z[k] (P = A^L, the zero-input transition over a chunk), then each chunk re-run
    from its entering state -- equal to one sequential pass (scipy.signal.sosfilt)."""
    sos = signal.butter(3, 300.0, btype="high", fs=30000.0, output="sos")
    ns, L = len(sos), 32
    rng = np.random.default_rng(0)
    x = np.cumsum(rng.normal(0, 10, 1000)) + 500.0   # drifting, offset: the filter must remove it
    zi = signal.sosfilt_zi(sos) * x[0]
    ref, _ = signal.sosfilt(sos, x, zi=zi)
    A = np.zeros((2 * ns, 2 * ns))
    for j in range(2 * ns):
        z = np.zeros((ns, 2))
        z.flat[j] = 1.0
        _cascade(sos, np.zeros(1), z)
        A[:, j] = z.ravel()
    P = np.linalg.matrix_power(A, L)
    chunks = [x[i:i + L] for i in range(0, len(x), L)]
    zs = []
    for c in chunks:
        z = np.zeros((ns, 2))
        _cascade(sos, c, z)
        zs.append(z.ravel())
    s = zi.ravel().copy()
    out, entering = [], []
    for c, z in zip(chunks, zs):
        entering.append(s.copy())
        out.append(_cascade(sos, c, s.reshape(ns, 2).copy()))
        s = P @ s + z
    np.testing.assert_allclose(np.concatenate(out), ref, rtol=0, atol=1e-9 * np.abs(ref).max())
    # the streaming kernel's warp scan over 32 chunks at a time: inclusive prefixes by
    # v_i += P^d v_(i-d) (d = 1, 2, 4, 8, 16), entering state of chunk q0 + i = P^i s0 + v_(i-1)
    Pw = [np.linalg.matrix_power(P, i) for i in range(33)]
    s0 = zi.ravel().copy()
    got = []
    for q0 in range(0, len(zs), 32):
        v = [zs[q] if q < len(zs) else np.zeros(2 * ns) for q in range(q0, q0 + 32)]
        d = 1
        while d < 32:
            v = [v[i] + (Pw[d] @ v[i - d] if i >= d else 0) for i in range(32)]
            d *= 2
        got += [Pw[i] @ s0 + (v[i - 1] if i else 0) for i in range(32) if q0 + i < len(zs)]
        s0 = Pw[32] @ s0 + v[31]
    np.testing.assert_allclose(np.array(got), np.array(entering), rtol=0, atol=1e-9 * np.abs(entering).max())


def test_oracle_filter_chunked_equals_whole():
    sos = ko.highpass_sos()
    x = np.random.default_rng(1).integers(-300, 300, (5000, 4)).astype(np.float64)
    whole, _ = ko.sos_highpass(x, sos)
    a, zf = ko.sos_highpass(x[:1777], sos)
    b, _ = ko.sos_highpass(x[1777:], sos, zi=zf)
    np.testing.assert_allclose(np.concatenate([a, b]), whole, rtol=0, atol=1e-10)
    # a constant input in its steady state gives zero output
    c, _ = ko.sos_highpass(np.full((100, 2), 123.0), sos)
    assert np.abs(c).max() < 1e-9


def test_oracle_stream_framing():
    """Window j of the padded stream is Kilosort's padded batch j (KS/io.py:584-637)."""
    data = np.random.default_rng(2).integers(-100, 100, (3 * 400 + 57, 3)).astype(np.int16)
    NT, nt = 400, 11
    P = ko.biquad_padded_stream(data, NT, nt)
    for j in range(ko.n_batches(data.shape[0], NT)):
        np.testing.assert_array_equal(P[j * NT: j * NT + NT + 2 * nt].T, ko.padded_batch(data, j, NT, nt))
    one = data[:300]
    np.testing.assert_array_equal(ko.biquad_padded_stream(one, NT, nt).T, ko.padded_batch(one, 0, NT, nt))


def test_open_rejects_bad_highpass_parameters(tmp_path):
    cfg = synth.SynthConfig(n_chan=32, n_units=8, n_samples=3000, whiten_batch=1000, whiten_batches=2, seed=3)
    rec = synth.make_recording(cfg)
    d = synth.write_oss_input(synth.build_oss_input(rec), tmp_path / "oss_input")
    lib = sorter.load_library()
    for kw in ({"highpass_mode": 2}, {"highpass_mode": 1, "highpass_hz": 20000.0},
               {"highpass_mode": 1, "sample_rate_hz": 0.0}):
        p = sorter.default_params(**kw)
        h = ct.c_void_p()
        assert lib.lss_open(str(d).encode(), ct.byref(p), ct.byref(h)) == 1, kw   # LSS_ERR_ARG
    p = sorter.default_params()
    assert (p.highpass_mode, p.highpass_hz, p.sample_rate_hz) == (0, 300.0, 30000.0)
