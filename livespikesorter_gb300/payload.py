"""Python mirror of ``include/lss_payload.h``: the per-batch spike message in the reference's wire
format (OnlineSpikesPayload serialized by cereal's binary archive,
src/Networking/onlineSpikesPayload.h:8-48).  Every call goes to ``liblss_gb300.so``."""
from __future__ import annotations

import ctypes as ct

import numpy as np

from .sorter import SPIKE_DTYPE, SorterError, load_library


class PayloadHeader(ct.Structure):
    _fields_ = [("recording_offset", ct.c_int64), ("stream_sample_ct", ct.c_int64), ("vrms", ct.c_double),
                ("p2p", ct.c_float), ("reserved", ct.c_int32), ("process_time", ct.c_int64),
                ("event_stream_sample_ct", ct.c_int64), ("predict_label", ct.c_int16), ("label", ct.c_int16),
                ("n_trials", ct.c_int16), ("n_correct", ct.c_int16), ("confidence", ct.c_double)]


HEADER_FIELDS = [f for f, _ in PayloadHeader._fields_ if f != "reserved"]


def _check(st, what):
    if st:
        raise SorterError(st, what)


def size(n_spikes: int, long_bytes: int = 4) -> int:
    n = ct.c_int64()
    _check(load_library().lss_payload_size(n_spikes, long_bytes, ct.byref(n)), "bad size arguments")
    return n.value


def serialize(spikes: np.ndarray, long_bytes: int = 4, **header) -> bytes:
    """The message of one batch: spikes (SPIKE_DTYPE records) and header fields by name."""
    lib = load_library()
    h = PayloadHeader()
    for k, v in header.items():
        if k not in HEADER_FIELDS:
            raise KeyError(k)
        setattr(h, k, v)
    sp = np.ascontiguousarray(spikes, dtype=SPIKE_DTYPE)
    out = np.zeros(size(len(sp), long_bytes), np.uint8)
    n = ct.c_int64()
    _check(lib.lss_payload_serialize(ct.byref(h), sp.ctypes.data if len(sp) else None, len(sp), long_bytes,
                                     out.ctypes.data, len(out), ct.byref(n)), "serialize failed")
    return out[:n.value].tobytes()


def parse(buf: bytes, long_bytes: int = 4):
    """(header dict, times int64, templates int64, amplitudes float32) of one message."""
    lib = load_library()
    b = np.frombuffer(buf, np.uint8)
    h = PayloadHeader()
    n = ct.c_int64()
    _check(lib.lss_payload_parse(b.ctypes.data, len(b), long_bytes, ct.byref(h), None, None, None, 0,
                                 ct.byref(n)), "malformed message")
    t = np.zeros(n.value, np.int64)
    k = np.zeros(n.value, np.int64)
    a = np.zeros(n.value, np.float32)
    _check(lib.lss_payload_parse(b.ctypes.data, len(b), long_bytes, ct.byref(h), t.ctypes.data, k.ctypes.data,
                                 a.ctypes.data, n.value, ct.byref(n)), "malformed message")
    return {f: getattr(h, f) for f in HEADER_FIELDS}, t, k, a


def batch_p2p(rows: np.ndarray) -> float:
    """Largest minus smallest raw sample of a batch [n_rows][n_chan] (the reference's P2P)."""
    r = np.ascontiguousarray(rows, dtype=np.int16)
    if r.ndim != 2:
        raise ValueError("rows must be [n_rows][n_chan]")
    v = ct.c_float()
    _check(load_library().lss_batch_p2p(r.ctypes.data, r.shape[0], r.shape[1], ct.byref(v)), "bad rows")
    return v.value
