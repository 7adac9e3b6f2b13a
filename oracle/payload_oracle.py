"""Restatement of the per-batch spike message's wire format -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` use this module, as the checker of ``lss_payload_serialize`` / ``lss_payload_parse``.

The message is the reference's OnlineSpikesPayload (src/Networking/onlineSpikesPayload.h:8-48)
written by cereal's BinaryOutputArchive (serialize<T>, src/Networking/SerializationHelpers.h:10-18):
every field in declaration order as its raw little-endian bytes, a std::vector as a uint64 element
count (CEREAL_SIZE_TYPE, External/cereal/macros.hpp:70) followed by its elements, no padding.
`long` is 4 bytes in the reference's Windows build, 8 on LP64.

Pinned against the reference's own cereal: ``payload_ref`` (oracle/payload_ref.cpp, built by
oracle/build_ref.py against External/cereal) serializes the same messages, and the bytes it
wrote are committed as tests/golden/payload_cereal.npz (tests/golden/make_payload_golden.py).
"""
from __future__ import annotations

import struct
import subprocess

import numpy as np

HEADER = ("recording_offset", "stream_sample_ct", "vrms", "p2p", "process_time", "event_stream_sample_ct",
          "predict_label", "label", "n_trials", "n_correct", "confidence")


def _long(long_bytes: int) -> str:
    return "<i" if long_bytes == 4 else "<q"


def _wrap(v: int, long_bytes: int) -> int:
    """The value a `long` of that width holds (low bits, two's complement)."""
    if long_bytes == 8:
        return int(v)
    v = int(v) & 0xFFFFFFFF
    return v - (1 << 32) if v >= 1 << 31 else v


def serialize(hdr: dict, times, templates, amps, long_bytes: int = 4) -> bytes:
    L = _long(long_bytes)
    h = {k: hdr.get(k, 0) for k in HEADER}
    n = len(times)
    out = [struct.pack(L, _wrap(h["recording_offset"], long_bytes)),
           struct.pack(L, _wrap(h["stream_sample_ct"], long_bytes)),
           struct.pack("<Q", n), b"".join(struct.pack(L, _wrap(t, long_bytes)) for t in times),
           struct.pack("<Q", n), b"".join(struct.pack(L, _wrap(t, long_bytes)) for t in templates),
           struct.pack("<Q", n), np.asarray(amps, "<f4").tobytes(),
           struct.pack("<d", h["vrms"]), struct.pack("<f", h["p2p"]),
           struct.pack(L, _wrap(h["process_time"], long_bytes)),
           struct.pack(L, _wrap(h["event_stream_sample_ct"], long_bytes)),
           struct.pack("<hhhh", h["predict_label"], h["label"], h["n_trials"], h["n_correct"]),
           struct.pack("<d", h["confidence"])]
    return b"".join(out)


def p2p(rows) -> float:
    """P2P_calc (src/SpikeSorter/OnlineSpikesV2.cu:1137-1146) as intended: the largest minus the
    smallest of the batch's float-converted samples."""
    r = np.asarray(rows).astype(np.float32)
    return float(np.float32(r.max()) - np.float32(r.min()))


def cereal_input(hdr: dict, times, templates, amps, long_bytes: int) -> bytes:
    """The stdin record of oracle/payload_ref.cpp for one message."""
    h = {k: hdr.get(k, 0) for k in HEADER}
    n = len(times)
    return b"".join([struct.pack("<i", long_bytes), struct.pack("<qq", h["recording_offset"], h["stream_sample_ct"]),
                     struct.pack("<Q", n), np.asarray(times, "<i8").tobytes(), np.asarray(templates, "<i8").tobytes(),
                     np.asarray(amps, "<f4").tobytes(), struct.pack("<d", h["vrms"]), struct.pack("<f", h["p2p"]),
                     struct.pack("<qq", h["process_time"], h["event_stream_sample_ct"]),
                     struct.pack("<hhhh", h["predict_label"], h["label"], h["n_trials"], h["n_correct"]),
                     struct.pack("<d", h["confidence"])])


def cereal_serialize(exe, hdr: dict, times, templates, amps, long_bytes: int) -> bytes:
    """The same message through the reference's cereal (oracle/_ref/payload_ref)."""
    r = subprocess.run([str(exe)], input=cereal_input(hdr, times, templates, amps, long_bytes),
                       capture_output=True, check=True)
    return r.stdout
