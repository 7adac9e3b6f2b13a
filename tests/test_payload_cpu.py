"""The per-batch spike message (include/lss_payload.h) without a GPU: the restated wire format
and the library's serializer against bytes written by the reference's own cereal
(tests/golden/payload_cereal.npz, made by tests/golden/make_payload_golden.py), parsing, the
errors of malformed messages, and the batch P2P."""
import numpy as np
import pytest

from livespikesorter_gb300 import payload, sorter
from oracle import payload_oracle as po

INT_FIELDS = {"recording_offset", "stream_sample_ct", "process_time", "event_stream_sample_ct", "predict_label",
              "label", "n_trials", "n_correct"}


@pytest.fixture(scope="module")
def golden(golden_dir):
    z = np.load(golden_dir / "payload_cereal.npz")
    out = []
    for i in range(int(z["n_cases"])):
        hdr = {k: (int(v) if k in INT_FIELDS else float(v)) for k, v in zip(po.HEADER, z[f"c{i}_header"])}
        out.append((hdr, z[f"c{i}_times"], z[f"c{i}_templates"], z[f"c{i}_amps"],
                    {lb: z[f"c{i}_bytes{lb}"].tobytes() for lb in (4, 8)}))
    return out


def _spikes(times, templates, amps):
    sp = np.zeros(len(times), sorter.SPIKE_DTYPE)
    sp["time"], sp["cluster"], sp["amp"] = times, templates, amps
    sp["tmpl"] = 999   # the message carries the final cluster, not the preclustered template
    return sp


def test_restated_format_matches_cereal(golden):
    for hdr, t, k, a, ref in golden:
        for lb in (4, 8):
            assert po.serialize(hdr, t, k, a, lb) == ref[lb]


def test_library_serializer_matches_cereal(golden):
    for hdr, t, k, a, ref in golden:
        for lb in (4, 8):
            got = payload.serialize(_spikes(t, k, a), lb, **hdr)
            assert got == ref[lb]
            assert payload.size(len(t), lb) == len(ref[lb])


def test_parse_round_trip(golden):
    for hdr, t, k, a, ref in golden:
        for lb in (4, 8):
            h, t2, k2, a2 = payload.parse(ref[lb], lb)
            wrap = (lambda v: v) if lb == 8 else (lambda v: ((np.asarray(v, np.int64) + 2**31) % 2**32) - 2**31)
            np.testing.assert_array_equal(t2, wrap(t))
            np.testing.assert_array_equal(k2, k)
            np.testing.assert_array_equal(a2, a)
            for f in po.HEADER:
                want = hdr[f]
                if lb == 4 and f in ("recording_offset", "stream_sample_ct", "process_time", "event_stream_sample_ct"):
                    want = int(wrap(want))
                assert h[f] == pytest.approx(want), f


def test_malformed_messages_are_refused(golden):
    hdr, t, k, a, ref = golden[2]
    b = ref[4]
    for bad in (b[:-1], b + b"\0", b[:10], b""):
        with pytest.raises(sorter.SorterError):
            payload.parse(bad, 4)
    # a Templates count one short of the others (its elements shifted accordingly)
    n = len(t)
    off = 8 + 8 + 4 * n                       # 2 longs + count + times
    tampered = bytearray(b)
    tampered[off:off + 8] = (n - 1).to_bytes(8, "little")
    with pytest.raises(sorter.SorterError):
        payload.parse(bytes(tampered), 4)
    with pytest.raises(sorter.SorterError):
        payload.parse(b, 8)                   # the wrong long width does not parse


def test_serializer_reports_the_size_it_needs():
    lib = sorter.load_library()
    import ctypes as ct
    sp = _spikes([1, 2, 3], [4, 5, 6], [1.0, 2.0, 3.0])
    h = payload.PayloadHeader()
    n = ct.c_int64()
    buf = np.zeros(10, np.uint8)
    st = lib.lss_payload_serialize(ct.byref(h), sp.ctypes.data, 3, 4, buf.ctypes.data, len(buf), ct.byref(n))
    assert st != 0 and n.value == payload.size(3, 4) == 68 + 3 * 12
    assert lib.lss_payload_size(3, 5, ct.byref(n)) != 0      # only 4- or 8-byte longs


def test_batch_p2p():
    rng = np.random.default_rng(1)
    for shape in ((1500, 384), (1, 1), (7, 3)):
        rows = rng.integers(-32768, 32768, shape).astype(np.int16)
        assert payload.batch_p2p(rows) == po.p2p(rows)
    assert payload.batch_p2p(np.full((4, 2), -7, np.int16)) == 0.0


def test_fresh_messages_against_cereal_when_the_reference_is_present():
    from oracle import build_ref
    exe = build_ref.build()
    if exe is None:
        pytest.skip("the reference checkout is absent: the committed golden bytes stand in")
    rng = np.random.default_rng(99)
    for n in (3, 64):
        t = rng.integers(-(1 << 40), 1 << 40, n)
        k = rng.integers(-1, 3000, n)
        a = rng.normal(0, 100, n).astype(np.float32)
        hdr = {"recording_offset": int(rng.integers(-(1 << 40), 1 << 40)), "p2p": 3.25, "process_time": 123}
        for lb in (4, 8):
            assert payload.serialize(_spikes(t, k, a), lb, **hdr) == po.cereal_serialize(exe, hdr, t, k, a, lb)
