"""Python mirror of the threshold-crossing detector's C ABI (``include/lss_threshold.h``).

``ThresholdCrossing`` follows the reference's second sorter (src/SpikeSorter/ThresholdCrossing.h:
17-93): built from per-channel means and medians and a threshold in units of the median, it takes
int16 rows and returns (time, channel, value) events, each push in the reference's order (channel,
then row).  Every call goes to ``liblss_gb300.so``; there is no Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from .sorter import SorterError, load_library

TC_ABI_VERSION = 1
TC_STAGES = ("h2d", "count", "offsets", "emit", "d2h")


class TcParams(ct.Structure):
    _fields_ = [("abi_version", ct.c_int32), ("device", ct.c_int32), ("n_chan", ct.c_int32),
                ("threshold_std", ct.c_float), ("max_rows", ct.c_int64), ("event_cap", ct.c_int64),
                ("profile", ct.c_int32), ("reserved", ct.c_int32 * 5)]


class TcEvent(ct.Structure):
    _fields_ = [("time", ct.c_int64), ("channel", ct.c_int32), ("value", ct.c_float)]


EVENT_DTYPE = np.dtype([("time", "<i8"), ("channel", "<i4"), ("value", "<f4")])
assert EVENT_DTYPE.itemsize == ct.sizeof(TcEvent)


def _f32(a, n):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.shape != (n,):
        raise ValueError(f"expected {n} values, got shape {a.shape}")
    return a


def int_thresholds(means, medians, threshold_std) -> np.ndarray:
    """Per-channel integer thresholds (host only; lss_tc_int_thresholds)."""
    lib = load_library()
    mu = np.ascontiguousarray(means, dtype=np.float32)
    md = _f32(medians, len(mu))
    out = np.zeros(len(mu), np.int32)
    st = lib.lss_tc_int_thresholds(len(mu), mu.ctypes.data, md.ctypes.data, ct.c_float(threshold_std),
                                   out.ctypes.data)
    if st:
        raise SorterError(st, (lib.lss_tc_last_error(None) or b"").decode())
    return out


def calibrate(rows):
    """(means, medians) of a block of int16 rows [n][C] (host only; lss_tc_calibrate)."""
    lib = load_library()
    r = np.ascontiguousarray(rows, dtype=np.int16)
    n, c = r.shape
    mu = np.zeros(c, np.float32)
    md = np.zeros(c, np.float32)
    st = lib.lss_tc_calibrate(r.ctypes.data, n, c, mu.ctypes.data, md.ctypes.data)
    if st:
        raise SorterError(st, (lib.lss_tc_last_error(None) or b"").decode())
    return mu, md


class ThresholdCrossing:
    """One threshold-crossing detector on one GPU (the reference's ``ThresholdCrossing``)."""

    def __init__(self, means, medians, threshold_std=3.0, device=0, max_rows=1500, event_cap=0, profile=0):
        self.lib = load_library()
        mu = np.ascontiguousarray(means, dtype=np.float32)
        md = _f32(medians, len(mu))
        p = TcParams()
        self.lib.lss_tc_default_params(ct.byref(p))
        p.device, p.n_chan, p.threshold_std = device, len(mu), threshold_std
        p.max_rows, p.event_cap, p.profile = max_rows, event_cap, profile
        self.params = p
        self.n_chan = len(mu)
        h = ct.c_void_p()
        st = self.lib.lss_tc_open(ct.byref(p), mu.ctypes.data, md.ctypes.data, ct.byref(h))
        if st:
            raise SorterError(st, (self.lib.lss_tc_last_error(None) or b"").decode())
        self.h = h
        self._buf = np.zeros(1 << 16, EVENT_DTYPE)

    def _check(self, st, allow=()):
        if st and st not in allow:
            raise SorterError(st, (self.lib.lss_tc_last_error(self.h) or b"").decode())
        return st

    def close(self):
        if getattr(self, "h", None):
            self.lib.lss_tc_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def push(self, rows, first_row_sample=0):
        r = np.ascontiguousarray(rows, dtype=np.int16)
        if r.ndim != 2 or r.shape[1] != self.n_chan:
            raise ValueError(f"rows must be [n][{self.n_chan}] int16")
        self._check(self.lib.lss_tc_push(self.h, r.ctypes.data, r.shape[0], first_row_sample))

    def push_device(self, ptr: int, n_rows: int, first_row_sample=0):
        """Rows already on the device: ptr = address of int16 [n_rows][n_chan]."""
        self._check(self.lib.lss_tc_push_device(self.h, ct.c_void_p(ptr), n_rows, first_row_sample))

    def poll(self, cap=None, allow_overflow=False):
        """Events waiting (blocking for the oldest push in flight when none are)."""
        if cap is not None and cap > len(self._buf):
            self._buf = np.zeros(cap, EVENT_DTYPE)
        n = ct.c_int64()
        want = len(self._buf) if cap is None else cap
        st = self._check(self.lib.lss_tc_poll(self.h, self._buf.ctypes.data, want, ct.byref(n)),
                         allow=(6,) if allow_overflow else ())
        out = self._buf[:n.value].copy()
        return (out, st) if allow_overflow else out

    def poll_all(self):
        """Every event of every push made so far, in order."""
        parts = []
        while True:
            pend = ct.c_int64()
            self._check(self.lib.lss_tc_pending(self.h, ct.byref(pend)))
            if pend.value == 0:
                break
            parts.append(self.poll(cap=max(pend.value, 1)))
        return np.concatenate(parts) if parts else np.zeros(0, EVENT_DTYPE)

    def thresholds(self):
        out = np.zeros(self.n_chan, np.int32)
        self._check(self.lib.lss_tc_thresholds(self.h, out.ctypes.data, self.n_chan))
        return out

    def cuda_stream(self) -> int:
        s = ct.c_void_p()
        self._check(self.lib.lss_tc_cuda_stream(self.h, ct.byref(s)))
        return s.value or 0

    def kernel_launches(self) -> int:
        n = ct.c_int64()
        self._check(self.lib.lss_tc_kernel_launches(self.h, ct.byref(n)))
        return n.value

    def stage_times(self):
        ms = (ct.c_double * len(TC_STAGES))()
        n = ct.c_int64()
        self._check(self.lib.lss_tc_stage_times(self.h, ms, len(TC_STAGES), ct.byref(n)))
        return dict(zip(TC_STAGES, list(ms))), n.value
