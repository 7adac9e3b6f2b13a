"""Learned proposal gate: Python mirror of ``include/lss_proposal.h``.

A 4-layer channel-local 1-D convolution network (16 channels in, 64 hidden, 7 taps, one logit per
sample) marks which (16-channel neighbourhood, 32-sample window) cells of a batch window may hold
a spike; a sorter with the gate set (``OnlineSorter.set_proposal``) lets the matching loop consider
template t at sample s only where the cell of t's peak channel and s is open.  The network is
trained on the device by the library's own forward / backward / Adam kernels
(``ProposalTrainer``), on labels that the plain matcher (the sorter without a gate) produces.

Every compute call goes to ``liblss_gb300.so``; there is no Python or CPU fallback.  PyTorch only
holds the whitened training windows in device memory.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from .sorter import STAGE_PREPROCESSED, SorterError, load_library

N_PARAMS = 65153
CHANNELS, HIDDEN, TAPS, WINDOW = 16, 64, 7, 32
SHAPES = ((HIDDEN, CHANNELS), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (1, HIDDEN))   # (out, in) per layer


class TrainParams(ct.Structure):
    _fields_ = [("device", ct.c_int32), ("max_examples", ct.c_int32), ("W", ct.c_int32), ("nt", ct.c_int32),
                ("lr", ct.c_float), ("beta1", ct.c_float), ("beta2", ct.c_float), ("eps", ct.c_float)]


def _err(lib, st, h=None):
    return SorterError(st, (lib.lss_prop_trainer_last_error(h) or b"").decode())


def n_windows(W: int, nt: int) -> int:
    """32-sample windows tiling a batch window's interior [nt, W - nt)."""
    return -(-(W - 2 * nt) // WINDOW)


def neighbourhoods(n_chan: int) -> np.ndarray:
    lib = load_library()
    n = ct.c_int32()
    st = lib.lss_prop_neighbourhoods(n_chan, ct.byref(n), None, 0)
    if st:
        raise SorterError(st, "bad channel count")
    out = np.zeros(n.value, np.int32)
    lib.lss_prop_neighbourhoods(n_chan, ct.byref(n), out.ctypes.data, len(out))
    return out


def template_owner(Wall3: np.ndarray) -> np.ndarray:
    """Neighbourhood of each template's peak channel, from Wall3 [T][K][C]."""
    lib = load_library()
    w = np.ascontiguousarray(Wall3, dtype=np.float32)
    T, K, C = w.shape
    out = np.zeros(T, np.int32)
    st = lib.lss_prop_template_owner(w.ctypes.data, T, K, C, out.ctypes.data)
    if st:
        raise SorterError(st, "bad Wall3")
    return out


def init_params(seed: int = 0, prior: float = 0.1) -> np.ndarray:
    """He-normal hidden layers; a small output layer whose bias is the logit of ``prior``."""
    rng = np.random.default_rng(seed)
    parts = []
    for li, (o, i) in enumerate(SHAPES):
        std = np.sqrt(2.0 / (i * TAPS)) if li < 3 else 0.01
        b = np.zeros(o)
        if li == 3:
            b[:] = np.log(prior / (1.0 - prior))
        parts += [rng.normal(0.0, std, o * i * TAPS), b]
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == N_PARAMS
    return p


def window_labels(samples, templates, owner, n_nbhd: int, W: int, nt: int) -> np.ndarray:
    """[n_nbhd, n_win] uint8: 1 where a spike (window sample, template) of the plain matcher falls
    in the window and its template's peak channel belongs to the neighbourhood."""
    lab = np.zeros((n_nbhd, n_windows(W, nt)), np.uint8)
    s = np.asarray(samples, np.int64)
    t = np.asarray(templates, np.int64)
    keep = (s >= nt) & (s < W - nt)
    lab[np.asarray(owner)[t[keep]], (s[keep] - nt) // WINDOW] = 1
    return lab


def dilated_logits(z: np.ndarray, dilate: int) -> np.ndarray:
    """Largest window logit within ``dilate`` windows (a cell is open after dilation exactly when
    this exceeds the threshold)."""
    out = np.array(z, copy=True)
    for d in range(1, dilate + 1):
        out[..., d:] = np.maximum(out[..., d:], z[..., :-d])
        out[..., :-d] = np.maximum(out[..., :-d], z[..., d:])
    return out


def choose_threshold(z: np.ndarray, labels: np.ndarray, dilate: int, recall: float) -> float:
    """Largest logit threshold that keeps at least ``recall`` of the labelled cells open."""
    zd = dilated_logits(z, dilate)[np.asarray(labels) > 0]
    if zd.size == 0:
        return float("inf")
    k = int(np.floor((1.0 - recall) * zd.size))
    return float(np.nextafter(np.float32(np.sort(zd)[k]), np.float32(-np.inf)))


class ProposalTrainer:
    """FP32 master parameters and Adam state on one GPU; examples gathered on the device."""

    def __init__(self, W: int, nt: int, max_examples: int = 128, device: int = 0, lr: float = 1e-3,
                 params: np.ndarray = None, seed: int = 0):
        self.lib = load_library()
        self.W, self.nt, self.max_examples = W, nt, max_examples
        self.n_win = n_windows(W, nt)
        p = TrainParams(device=device, max_examples=max_examples, W=W, nt=nt, lr=lr)
        init = np.ascontiguousarray(init_params(seed) if params is None else params, dtype=np.float32)
        if init.size != N_PARAMS:
            raise ValueError(f"expected {N_PARAMS} parameters")
        h = ct.c_void_p()
        st = self.lib.lss_prop_trainer_open(ct.byref(p), init.ctypes.data, ct.byref(h))
        if st:
            raise _err(self.lib, st)
        self.h = h
        self.steps = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.lss_prop_trainer_close(self.h)
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

    def _check(self, st):
        if st:
            raise _err(self.lib, st, self.h)

    def _args(self, z, pairs, labels=None):
        import torch
        if not (isinstance(z, torch.Tensor) and z.is_cuda and z.dtype == torch.float32 and z.dim() == 3
                and z.is_contiguous() and z.shape[1] == self.W):
            raise ValueError("z must be a contiguous float32 CUDA tensor [n_windows, W, C]")
        torch.cuda.synchronize(z.device)
        pr = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        lab = None
        if labels is not None:
            lab = np.ascontiguousarray(labels, dtype=np.uint8).reshape(len(pr), self.n_win)
        return z.data_ptr(), z.shape[0], z.shape[2], pr, lab

    def step(self, z, pairs, labels) -> float:
        zp, n, C, pr, lab = self._args(z, pairs, labels)
        loss = ct.c_float()
        self._check(self.lib.lss_prop_train_step(self.h, zp, n, C, pr.ctypes.data, lab.ctypes.data, len(pr),
                                                 ct.byref(loss)))
        self.steps += 1
        return loss.value

    def loss_grad(self, z, pairs, labels):
        zp, n, C, pr, lab = self._args(z, pairs, labels)
        loss = ct.c_float()
        g = np.zeros(N_PARAMS, np.float32)
        self._check(self.lib.lss_prop_loss_grad(self.h, zp, n, C, pr.ctypes.data, lab.ctypes.data, len(pr),
                                                ct.byref(loss), g.ctypes.data))
        return loss.value, g

    def forward(self, z, pairs):
        """(per-sample logits [E, W], window logits [E, n_win])."""
        zp, n, C, pr, _ = self._args(z, pairs)
        lg = np.zeros((len(pr), self.W), np.float32)
        zw = np.zeros((len(pr), self.n_win), np.float32)
        self._check(self.lib.lss_prop_forward(self.h, zp, n, C, pr.ctypes.data, len(pr), lg.ctypes.data,
                                              zw.ctypes.data))
        return lg, zw

    @property
    def params(self) -> np.ndarray:
        p = np.zeros(N_PARAMS, np.float32)
        self._check(self.lib.lss_prop_get_params(self.h, p.ctypes.data))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != N_PARAMS:
            raise ValueError(f"expected {N_PARAMS} parameters")
        self._check(self.lib.lss_prop_set_params(self.h, p.ctypes.data))
        self.steps = 0


# ----------------------------------------------------------------------------- training set

def batch_windows(data: np.ndarray, first: int, n: int, NT: int, nt: int) -> np.ndarray:
    """Windows j = first .. first+n-1 of a recording [N][C] (rows j*NT .. j*NT + NT + 2nt)."""
    W = NT + 2 * nt
    return np.stack([data[j * NT:j * NT + W] for j in range(first, first + n)])


def plain_labels(sorter, windows: np.ndarray, owner: np.ndarray, n_nbhd: int):
    """Sort the windows with ``sorter`` (no gate set) and turn its spikes into cell labels
    [n][n_nbhd][n_win]; also returns the spikes of each window."""
    info = sorter.info
    W, nt = windows.shape[1], info.nt
    spikes = sorter.sort_windows(windows)
    labs = []
    for sp in spikes:
        s = sp["time"] + nt // 2 - info.nt0min          # window sample (the windows start at 0)
        labs.append(window_labels(s, sp["tmpl"], owner, n_nbhd, W, nt))
    return np.stack(labs), spikes


def whitened(sorter, windows: np.ndarray):
    """Whitened windows [n][W][C] as a CUDA tensor (the sorter's preprocessing, one per call)."""
    import torch
    Z = np.stack([sorter.debug_stage(w, STAGE_PREPROCESSED) for w in windows])
    return torch.from_numpy(Z).cuda()


def all_pairs(n_windows_: int, starts: np.ndarray) -> np.ndarray:
    """(window, neighbourhood start) of every example, windows major."""
    j = np.repeat(np.arange(n_windows_, dtype=np.int32), len(starts))
    return np.stack([j, np.tile(starts.astype(np.int32), n_windows_)], 1)


def train(trainer: ProposalTrainer, z, labels: np.ndarray, starts: np.ndarray, steps: int, batch: int = 64,
          seed: int = 0):
    """Adam on random minibatches of (window, neighbourhood) examples; returns the losses."""
    rng = np.random.default_rng(seed)
    pairs = all_pairs(labels.shape[0], starts)
    flat = labels.reshape(-1, labels.shape[-1])
    batch = min(batch, trainer.max_examples, len(pairs))
    losses = []
    for _ in range(steps):
        idx = rng.choice(len(pairs), batch, replace=False)
        losses.append(trainer.step(z, pairs[idx], flat[idx]))
    return np.asarray(losses)


def window_logits(trainer: ProposalTrainer, z, starts: np.ndarray) -> np.ndarray:
    """[n_windows][n_nbhd][n_win] window logits of every cell (FP32 weights)."""
    pairs = all_pairs(z.shape[0], starts)
    out = []
    for i in range(0, len(pairs), trainer.max_examples):
        out.append(trainer.forward(z, pairs[i:i + trainer.max_examples])[1])
    return np.concatenate(out).reshape(z.shape[0], len(starts), -1)
