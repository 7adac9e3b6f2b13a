"""Python mirror of the sorter's C ABI (``include/lss_gb300.h``) over ctypes.  The library's
other functions are declared here too: threshold crossing (``include/lss_threshold.h``, wrapped
in ``threshold.py``), the learned proposal gate (``include/lss_proposal.h``, ``proposal.py``) and
the per-batch spike message (``include/lss_payload.h``, ``payload.py``).

``OnlineSorter`` follows the reference's sorter surface (src/SpikeSorter/OnlineSpikesV2.h:29-34):
construct it on an ``oss_input/`` directory, push int16 samples, and poll the sorted spikes.
Every call goes to ``liblss_gb300.so``; there is no Python or CPU fallback -- importing works
without a GPU, but opening a sorter without a CUDA device raises ``SorterError``.
"""
from __future__ import annotations

import ctypes as ct
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("LSS_GB300_LIB", _PKG / "lib" / "liblss_gb300.so"))

ABI_VERSION = 3
MAX_PCFEAT = 64
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_IO", 3: "ERR_FORMAT", 4: "ERR_CUDA", 5: "ERR_NOMEM",
          6: "ERR_OVERFLOW", 7: "ERR_STATE", 8: "ERR_INTERNAL"}
STAGE_PREPROCESSED, STAGE_SCORES, STAGE_RESIDUAL = 1, 2, 3


class Params(ct.Structure):
    _fields_ = [("abi_version", ct.c_int32), ("device", ct.c_int32), ("batch_samples", ct.c_int32),
                ("max_iters", ct.c_int32), ("group_batches", ct.c_int32), ("n_chan_in", ct.c_int32),
                ("hp_half_taps", ct.c_int32), ("dedup", ct.c_int32), ("th_override", ct.c_float),
                ("spike_cap", ct.c_int32), ("mem_budget", ct.c_int64), ("profile", ct.c_int32),
                ("match_variant", ct.c_int32), ("gemm_path", ct.c_int32), ("cluster_rule", ct.c_int32),
                ("cluster_radius_um", ct.c_float), ("match_keep", ct.c_int32),
                ("highpass_mode", ct.c_int32), ("highpass_hz", ct.c_float), ("sample_rate_hz", ct.c_float),
                ("match_keep_wide", ct.c_int32), ("match_keep_crowd", ct.c_float)]


class Spike(ct.Structure):
    _fields_ = [("time", ct.c_int64), ("tmpl", ct.c_int32), ("cluster", ct.c_int32), ("amp", ct.c_float),
                ("x", ct.c_float), ("y", ct.c_float), ("batch", ct.c_int32), ("n_feat", ct.c_int32),
                ("iter", ct.c_int32), ("pcfeat", ct.c_float * MAX_PCFEAT)]


class Info(ct.Structure):
    _fields_ = [("C", ct.c_int32), ("T", ct.c_int32), ("T_final", ct.c_int32), ("K", ct.c_int32),
                ("nt", ct.c_int32), ("nC", ct.c_int32), ("nt0min", ct.c_int32), ("dup_bins", ct.c_int32),
                ("th", ct.c_float), ("NT", ct.c_int32), ("W", ct.c_int32), ("group_batches", ct.c_int32),
                ("device_bytes", ct.c_int64), ("batches_done", ct.c_int64), ("spikes_done", ct.c_int64)]


SPIKE_DTYPE = np.dtype([("time", "<i8"), ("tmpl", "<i4"), ("cluster", "<i4"), ("amp", "<f4"), ("x", "<f4"),
                        ("y", "<f4"), ("batch", "<i4"), ("n_feat", "<i4"), ("iter", "<i4"),
                        ("pcfeat", "<f4", (MAX_PCFEAT,))])
assert SPIKE_DTYPE.itemsize == ct.sizeof(Spike)

# every function declared in include/lss_gb300.h: name -> (restype, argtypes)
_P = ct.POINTER
_SIGS = {
    "lss_default_params": (ct.c_int, [_P(Params)]),
    "lss_open": (ct.c_int, [ct.c_char_p, _P(Params), _P(ct.c_void_p)]),
    "lss_get_info": (ct.c_int, [ct.c_void_p, _P(Info)]),
    "lss_validate_oss_input": (ct.c_int, [ct.c_char_p, _P(Info)]),
    "lss_push_batch": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int64, ct.c_int64]),
    "lss_flush": (ct.c_int, [ct.c_void_p]),
    "lss_poll": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int64, _P(ct.c_int64)]),
    "lss_pending": (ct.c_int, [ct.c_void_p, _P(ct.c_int64)]),
    "lss_close": (ct.c_int, [ct.c_void_p]),
    "lss_last_error": (ct.c_char_p, [ct.c_void_p]),
    "lss_sort_windows": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int32, ct.c_int32, ct.c_void_p, ct.c_int64,
                                    ct.c_void_p]),
    "lss_debug_stage": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int32, ct.c_int32, ct.c_void_p, ct.c_int64]),
    "lss_kernel_launches": (ct.c_int, [ct.c_void_p, _P(ct.c_int64)]),
    "lss_push_device_span": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int64, ct.c_int64]),
    "lss_cuda_stream": (ct.c_int, [ct.c_void_p, _P(ct.c_void_p)]),
    "lss_stage_times": (ct.c_int, [ct.c_void_p, _P(ct.c_double), ct.c_int32, _P(ct.c_int64)]),
    "lss_butter_highpass_sos": (ct.c_int, [ct.c_int32, ct.c_double, ct.c_double, _P(ct.c_double), ct.c_int32,
                                           _P(ct.c_int32)]),
    "lss_match_noalloc": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_float,
                                     ct.c_int32, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_void_p,
                                     ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int32, ct.c_void_p]),
}
# include/lss_threshold.h (threshold-crossing detector; Python side in threshold.py)
_SIGS.update({
    "lss_tc_default_params": (ct.c_int, [ct.c_void_p]),
    "lss_tc_int_thresholds": (ct.c_int, [ct.c_int32, ct.c_void_p, ct.c_void_p, ct.c_float, ct.c_void_p]),
    "lss_tc_calibrate": (ct.c_int, [ct.c_void_p, ct.c_int64, ct.c_int32, ct.c_void_p, ct.c_void_p]),
    "lss_tc_open": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, _P(ct.c_void_p)]),
    "lss_tc_push": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int64, ct.c_int64]),
    "lss_tc_push_device": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int64, ct.c_int64]),
    "lss_tc_poll": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int64, _P(ct.c_int64)]),
    "lss_tc_pending": (ct.c_int, [ct.c_void_p, _P(ct.c_int64)]),
    "lss_tc_thresholds": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int32]),
    "lss_tc_cuda_stream": (ct.c_int, [ct.c_void_p, _P(ct.c_void_p)]),
    "lss_tc_kernel_launches": (ct.c_int, [ct.c_void_p, _P(ct.c_int64)]),
    "lss_tc_stage_times": (ct.c_int, [ct.c_void_p, _P(ct.c_double), ct.c_int32, _P(ct.c_int64)]),
    "lss_tc_close": (ct.c_int, [ct.c_void_p]),
    "lss_tc_last_error": (ct.c_char_p, [ct.c_void_p]),
})
# include/lss_proposal.h (learned proposal gate; Python side in proposal.py)
_SIGS.update({
    "lss_prop_neighbourhoods": (ct.c_int, [ct.c_int32, _P(ct.c_int32), ct.c_void_p, ct.c_int32]),
    "lss_prop_template_owner": (ct.c_int, [ct.c_void_p, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_void_p]),
    "lss_prop_trainer_open": (ct.c_int, [ct.c_void_p, ct.c_void_p, _P(ct.c_void_p)]),
    "lss_prop_trainer_close": (ct.c_int, [ct.c_void_p]),
    "lss_prop_trainer_last_error": (ct.c_char_p, [ct.c_void_p]),
    "lss_prop_train_step": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int32, ct.c_int32, ct.c_void_p, ct.c_void_p,
                                       ct.c_int32, _P(ct.c_float)]),
    "lss_prop_loss_grad": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int32, ct.c_int32, ct.c_void_p, ct.c_void_p,
                                      ct.c_int32, _P(ct.c_float), ct.c_void_p]),
    "lss_prop_forward": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int32, ct.c_int32, ct.c_void_p, ct.c_int32,
                                    ct.c_void_p, ct.c_void_p]),
    "lss_prop_get_params": (ct.c_int, [ct.c_void_p, ct.c_void_p]),
    "lss_prop_set_params": (ct.c_int, [ct.c_void_p, ct.c_void_p]),
    "lss_set_proposal": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_float, ct.c_int32]),
    "lss_proposal_stats": (ct.c_int, [ct.c_void_p, _P(ct.c_int64), _P(ct.c_int64)]),
})
# include/lss_payload.h (the per-batch spike message; Python side in payload.py)
_SIGS.update({
    "lss_payload_size": (ct.c_int, [ct.c_int64, ct.c_int32, _P(ct.c_int64)]),
    "lss_payload_serialize": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int64, ct.c_int32, ct.c_void_p, ct.c_int64,
                                         _P(ct.c_int64)]),
    "lss_payload_parse": (ct.c_int, [ct.c_void_p, ct.c_int64, ct.c_int32, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                     ct.c_void_p, ct.c_int64, _P(ct.c_int64)]),
    "lss_batch_p2p": (ct.c_int, [ct.c_void_p, ct.c_int64, ct.c_int32, _P(ct.c_float)]),
})
# template subsetting (Python side in subset.py; spec pointers are lss_subset_spec)
_SIGS.update({
    "lss_subset_default_spec": (None, [ct.c_void_p]),
    "lss_subset_plan": (ct.c_int, [ct.c_char_p, ct.c_void_p, _P(ct.c_int32), ct.c_int32, _P(ct.c_int32)]),
    "lss_subset_write": (ct.c_int, [ct.c_char_p, ct.c_char_p, ct.c_void_p]),
})
STAGES = ("h2d", "colsum", "car", "highpass", "whiten", "basis_conv", "project", "match", "features", "d2h")

_lib = None


def load_library(path=None) -> ct.CDLL:
    """Load liblss_gb300.so (building it first when it is missing and nvcc is available)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        from . import build
        build.build()
    lib = ct.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class SorterError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def validate_oss_input(oss_dir) -> Info:
    """Check an oss_input/ directory on the host (no GPU): lss_open's loader and shape checks.
    Returns its dimensions; raises SorterError with lss_open's status for a bad directory."""
    lib = load_library()
    info = Info()
    st = lib.lss_validate_oss_input(str(oss_dir).encode(), ct.byref(info))
    if st:
        raise SorterError(st, (lib.lss_last_error(None) or b"").decode())
    return info


def default_params(**kw) -> Params:
    lib = load_library()
    p = Params()
    lib.lss_default_params(ct.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def butter_highpass_sos(order: int = 3, cutoff_hz: float = 300.0, fs_hz: float = 30000.0) -> np.ndarray:
    """The library's second-order sections [n, 6] of the Butterworth high-pass of highpass_mode 1."""
    lib = load_library()
    sos = np.zeros((4, 6), np.float64)
    n = ct.c_int32()
    st = lib.lss_butter_highpass_sos(order, cutoff_hz, fs_hz, sos.ctypes.data_as(_P(ct.c_double)), 4, ct.byref(n))
    if st != 0:
        raise SorterError(st, "lss_butter_highpass_sos: bad arguments")
    return sos[: n.value].copy()


class OnlineSorter:
    """One probe stream on one GPU (the reference's ``OnlineSpikesV2`` instance)."""

    def __init__(self, oss_dir, **params):
        self.lib = load_library()
        self.params = default_params(**params)
        h = ct.c_void_p()
        st = self.lib.lss_open(str(oss_dir).encode(), ct.byref(self.params), ct.byref(h))
        if st != 0:
            raise SorterError(st, (self.lib.lss_last_error(None) or b"").decode())
        self.h = h
        self.info = Info()
        self.lib.lss_get_info(self.h, ct.byref(self.info))

    # -- helpers -------------------------------------------------------------------------
    def _check(self, st: int):
        if st != 0:
            raise SorterError(st, (self.lib.lss_last_error(self.h) or b"").decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.lss_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_info(self) -> Info:
        self.lib.lss_get_info(self.h, ct.byref(self.info))
        return self.info

    def cuda_stream(self) -> int:
        v = ct.c_void_p()
        self._check(self.lib.lss_cuda_stream(self.h, ct.byref(v)))
        return v.value or 0

    def stage_times(self):
        ms = (ct.c_double * len(STAGES))()
        n = ct.c_int64()
        self._check(self.lib.lss_stage_times(self.h, ms, len(STAGES), ct.byref(n)))
        return dict(zip(STAGES, list(ms))), n.value

    def push_device_span(self, dev_ptr: int, n_batches: int, first_row_sample: int = 0):
        self._check(self.lib.lss_push_device_span(self.h, ct.c_void_p(dev_ptr), int(n_batches), int(first_row_sample)))

    def kernel_launches(self) -> int:
        n = ct.c_int64()
        self._check(self.lib.lss_kernel_launches(self.h, ct.byref(n)))
        return n.value

    # -- learned proposal gate (include/lss_proposal.h) ----------------------------------
    def set_proposal(self, params, logit_threshold: float = 0.0, dilate: int = 1):
        """Gate the matching loop with a trained proposal network (None removes the gate)."""
        if params is None:
            self._check(self.lib.lss_set_proposal(self.h, None, ct.c_float(0.0), 0))
            return
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != 65153:
            raise ValueError("expected 65153 parameters")
        self._check(self.lib.lss_set_proposal(self.h, p.ctypes.data, ct.c_float(logit_threshold), dilate))

    def proposal_stats(self):
        """(cells evaluated, cells left open) since the gate was set."""
        c, o = ct.c_int64(), ct.c_int64()
        self._check(self.lib.lss_proposal_stats(self.h, ct.byref(c), ct.byref(o)))
        return c.value, o.value

    # -- streaming -----------------------------------------------------------------------
    def push(self, samples: np.ndarray, stream_sample_ct: int = -1):
        x = np.ascontiguousarray(samples, dtype=np.int16)
        if x.ndim != 2:
            raise ValueError("samples must be [n_samples, n_chan]")
        self._check(self.lib.lss_push_batch(self.h, x.ctypes.data, x.shape[0], int(stream_sample_ct)))

    def flush(self):
        self._check(self.lib.lss_flush(self.h))

    def poll(self, cap: int = 1 << 16, allow_overflow: bool = False, out: np.ndarray = None) -> np.ndarray:
        """Finished spikes (at most cap, or len(out) when a reusable buffer is given)."""
        if out is None:
            out = np.zeros(cap, SPIKE_DTYPE)
        cap = len(out)
        n = ct.c_int64()
        st = self.lib.lss_poll(self.h, out.ctypes.data, cap, ct.byref(n))
        if not (allow_overflow and st == 6):
            self._check(st)
        return out[: n.value]

    def pending(self) -> int:
        n = ct.c_int64()
        self._check(self.lib.lss_pending(self.h, ct.byref(n)))
        return n.value

    def poll_all(self) -> np.ndarray:
        n = self.pending()
        return self.poll(max(n, 1))

    def sort_stream(self, data: np.ndarray, chunk: int = 0) -> np.ndarray:
        """Push a whole recording (optionally in chunks), flush, and return every spike."""
        chunk = chunk or data.shape[0]
        outs = []
        for i in range(0, data.shape[0], chunk):
            self.push(data[i:i + chunk])
            outs.append(self.poll(1 << 14).copy())
        self.flush()
        outs.append(self.poll_all())
        return np.concatenate(outs)

    # -- explicit windows --------------------------------------------------------------------
    def sort_windows(self, windows: np.ndarray, cap: int = 0):
        w = np.ascontiguousarray(windows, dtype=np.int16)
        if w.ndim == 2:
            w = w[None]
        n, W, _ = w.shape
        cap = cap or max(4096, 8 * W) * n
        out = np.zeros(cap, SPIKE_DTYPE)
        counts = np.zeros(n, np.int64)
        self._check(self.lib.lss_sort_windows(self.h, w.ctypes.data, n, W, out.ctypes.data, cap, counts.ctypes.data))
        res, o = [], 0
        for c in counts:
            res.append(out[o:o + c])
            o += c
        return res

    def debug_stage(self, window: np.ndarray, stage: int) -> np.ndarray:
        w = np.ascontiguousarray(window, dtype=np.int16)
        W = w.shape[0]
        cols = self.info.T if stage == STAGE_SCORES else self.info.C
        out = np.zeros((W, cols), np.float32)
        self._check(self.lib.lss_debug_stage(self.h, w.ctypes.data, W, stage, out.ctypes.data, out.size))
        return out


def header_functions(header=None):
    """Names of the functions declared in the C headers (include/*.h, or the one given)."""
    import re
    hs = [Path(header)] if header else sorted((_PKG.parent / "include").glob("*.h"))
    names = set()
    for h in hs:
        names |= set(re.findall(r"^\s*(?:int|void|const char\*)\s+(lss_\w+)\s*\(", h.read_text(), re.M))
    return sorted(names)
