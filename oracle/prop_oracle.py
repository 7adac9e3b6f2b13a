"""CPU restatement of the learned proposal gate -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` import this module, as the checker of the CUDA gate (``csrc/proposal.cu``); the
product path never calls it.

The gate is this project's own component, not a reference function: the reference has no
learned proposal stage (its matcher scores every template at every sample,
src/SpikeSorter/OnlineSpikesV2.cu:903-1001).  **Parity unpinned**: there is no reference
implementation to pin against; this restatement is pinned instead by central finite differences
of its own loss (``tests/test_proposal_cpu.py``), and the CUDA kernels are checked against it.

Definitions (float64 here):

* A neighbourhood is 16 consecutive channels; starts every 8 channels, the last one ending at the
  last channel (``neighbourhood_starts``).  Channels past C read as 0 when C < 16.
* The network maps x [16][L] (whitened samples of one neighbourhood, channel-major) to one logit
  per sample: conv(16->64) ReLU, conv(64->64) ReLU, conv(64->64) ReLU, conv(64->1); every conv has
  7 taps, 'same' zero padding (out[o][l] = b[o] + sum_i sum_k w[o][i][k] * x[i][l + k - 3]).
* A window is 32 samples of a batch window's interior [nt, W - nt); its logit is the max of its
  samples' logits (the first maximum for the gradient); its label is 1 when the plain matcher
  placed a spike at a sample of the window whose template's peak channel the neighbourhood owns.
* Loss: mean over (example, window) of softplus(z) - y * z (binary cross-entropy on logits).
* A channel is owned by the neighbourhood whose centre (start + 7.5) is nearest, ties to the
  lower; a template by the owner of its peak channel (largest sum_k Wall3[t, k, c]^2).
* Gate: a (neighbourhood, window) cell is open when its window logit exceeds the threshold;
  dilation d opens the cells d windows either side of an open one; the matcher considers template
  t at interior sample s only when the cell (owner(t), (s - nt) // 32) is open.
"""
from __future__ import annotations

import numpy as np

NBC, HID, TAPS, WIN = 16, 64, 7, 32
PAD = TAPS // 2
SHAPES = ((HID, NBC), (HID, HID), (HID, HID), (1, HID))     # (out, in) channels per layer


def param_count() -> int:
    return sum(o * i * TAPS + o for o, i in SHAPES)


def offsets():
    """[(w_offset, b_offset)] of each layer in the flat parameter vector (w then b per layer)."""
    out, p = [], 0
    for o, i in SHAPES:
        out.append((p, p + o * i * TAPS))
        p += o * i * TAPS + o
    return out


def unpack(params):
    params = np.asarray(params)
    layers = []
    for (o, i), (wo, bo) in zip(SHAPES, offsets()):
        layers.append((params[wo:wo + o * i * TAPS].reshape(o, i, TAPS), params[bo:bo + o]))
    return layers


# ----------------------------------------------------------------------------- geometry

def neighbourhood_starts(n_chan: int) -> np.ndarray:
    if n_chan <= NBC:
        return np.zeros(1, np.int32)
    s = list(range(0, n_chan - NBC + 1, NBC // 2))
    if s[-1] != n_chan - NBC:
        s.append(n_chan - NBC)
    return np.asarray(s, np.int32)


def channel_owner(n_chan: int) -> np.ndarray:
    centre = neighbourhood_starts(n_chan).astype(np.float64) + (NBC - 1) / 2.0
    d = np.abs(np.arange(n_chan)[:, None] - centre[None, :])
    return d.argmin(1).astype(np.int32)          # argmin takes the first (lower) on ties


def template_owner(Wall3: np.ndarray) -> np.ndarray:
    energy = (np.asarray(Wall3, np.float64) ** 2).sum(1)          # [T, C]
    return channel_owner(Wall3.shape[2])[energy.argmax(1)]


def n_windows(W: int, nt: int) -> int:
    return -(-(W - 2 * nt) // WIN)


# ----------------------------------------------------------------------------- network

def conv_same(x, w, b):
    """x [E, I, L], w [O, I, TAPS], b [O] -> [E, O, L]."""
    E, I, L = x.shape
    xp = np.zeros((E, I, L + 2 * PAD), x.dtype)
    xp[:, :, PAD:PAD + L] = x
    out = np.broadcast_to(b[None, :, None], (E, w.shape[0], L)).astype(np.float64).copy()
    for k in range(TAPS):
        out += np.einsum("oi,eil->eol", w[:, :, k], xp[:, :, k:k + L], optimize=True)
    return out


def forward(params, x):
    """-> ([a1, a2, a3] post-ReLU activations, logits [E, L])."""
    layers = unpack(np.asarray(params, np.float64))
    a = np.asarray(x, np.float64)
    acts = []
    for li, (w, b) in enumerate(layers):
        a = conv_same(a, w, b)
        if li < 3:
            a = np.maximum(a, 0.0)
            acts.append(a)
    return acts, a[:, 0, :]


def window_max(logit, W: int, nt: int):
    """(z [E, n_win], argmax sample [E, n_win]) over the interior windows."""
    nw = n_windows(W, nt)
    E = logit.shape[0]
    z = np.empty((E, nw))
    idx = np.empty((E, nw), np.int64)
    for w in range(nw):
        lo, hi = nt + WIN * w, min(nt + WIN * (w + 1), W - nt)
        seg = logit[:, lo:hi]
        a = seg.argmax(1)
        idx[:, w] = lo + a
        z[:, w] = seg[np.arange(E), a]
    return z, idx


def softplus(z):
    return np.maximum(z, 0.0) + np.log1p(np.exp(-np.abs(z)))


def loss_and_grad(params, x, labels, W: int, nt: int, argmax=None):
    """Mean binary cross-entropy of the window logits and its gradient (flat, params' layout).
    ``argmax`` [E, n_win] (optional) names the sample each window's maximum is taken at, for a
    comparison with a device whose FP32 logits may order near-equal samples differently."""
    layers = unpack(np.asarray(params, np.float64))
    x = np.asarray(x, np.float64)
    acts, logit = forward(params, x)
    z, idx = window_max(logit, W, nt)
    if argmax is not None:
        idx = np.asarray(argmax, np.int64)
        z = np.take_along_axis(logit, idx, axis=1)
    y = np.asarray(labels, np.float64)
    n = z.size
    loss = float((softplus(z) - y * z).sum() / n)
    dz = (1.0 / (1.0 + np.exp(-z)) - y) / n
    E, L = logit.shape
    g = np.zeros((E, 1, L))
    np.put_along_axis(g[:, 0, :], idx, dz, axis=1)
    ins = [x] + acts
    grads = [None] * 4
    for li in range(3, -1, -1):
        w, _ = layers[li]
        a_in = ins[li]
        ap = np.zeros((E, a_in.shape[1], L + 2 * PAD))
        ap[:, :, PAD:PAD + L] = a_in
        gw = np.stack([np.einsum("eol,eil->oi", g, ap[:, :, k:k + L], optimize=True) for k in range(TAPS)], -1)
        grads[li] = (gw, g.sum((0, 2)))
        if li > 0:
            # d/d a_in[i][l] = sum_o sum_k w[o][i][k] g[o][l - k + 3], through the previous ReLU
            gp = np.zeros((E, g.shape[1], L + 2 * PAD))
            gp[:, :, PAD:PAD + L] = g
            gi = np.zeros((E, a_in.shape[1], L))
            for k in range(TAPS):
                gi += np.einsum("oi,eol->eil", w[:, :, k], gp[:, :, 2 * PAD - k:2 * PAD - k + L], optimize=True)
            g = gi * (a_in > 0)
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, flat


def adam_step(params, m, v, grad, step: int, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (step counts from 1); float32 in and out, like the device's buffers."""
    p = np.asarray(params, np.float32)
    g = np.asarray(grad, np.float32)
    m = np.float32(b1) * m + np.float32(1 - b1) * g
    v = np.float32(b2) * v + np.float32(1 - b2) * g * g
    c1 = np.float32(1.0 / (1.0 - b1 ** step))
    c2 = np.float32(1.0 / (1.0 - b2 ** step))
    p = p - np.float32(lr) * (m * c1) / (np.sqrt(v * c2) + np.float32(eps))
    return p.astype(np.float32), m.astype(np.float32), v.astype(np.float32)


# ----------------------------------------------------------------------------- data and gate

def gather_examples(Z, pairs):
    """Z [n_win_batches, W, C] time-major; pairs [E, 2] = (window, neighbourhood start) -> [E, 16, W]."""
    Z = np.asarray(Z)
    E = len(pairs)
    nw, W, C = Z.shape
    x = np.zeros((E, NBC, W), np.float32)
    for e, (j, c0) in enumerate(pairs):
        c1 = min(C, c0 + NBC)
        x[e, :c1 - c0, :] = Z[j, :, c0:c1].T
    return x


def window_labels(samples, templates, owner_t, n_nbhd: int, W: int, nt: int) -> np.ndarray:
    """[n_nbhd, n_win] uint8 labels of one batch window from its spikes (sample, template)."""
    lab = np.zeros((n_nbhd, n_windows(W, nt)), np.uint8)
    s = np.asarray(samples, np.int64)
    t = np.asarray(templates, np.int64)
    keep = (s >= nt) & (s < W - nt)
    lab[owner_t[t[keep]], (s[keep] - nt) // WIN] = 1
    return lab


def open_cells(z, threshold: float, dilate: int = 0) -> np.ndarray:
    """z [..., n_win] window logits -> open mask (z > threshold, dilated along windows)."""
    m = np.asarray(z) > threshold
    if dilate:
        out = m.copy()
        for d in range(1, dilate + 1):
            out[..., d:] |= m[..., :-d]
            out[..., :-d] |= m[..., d:]
        m = out
    return m


def allowed_scores(open_mask, owner_t, W: int, nt: int) -> np.ndarray:
    """[W, T] bool: the matcher may use score (s, t); samples outside the interior stay allowed."""
    T = len(owner_t)
    a = np.ones((W, T), bool)
    s = np.arange(nt, W - nt)
    a[nt:W - nt, :] = open_mask[np.asarray(owner_t)[None, :], ((s - nt) // WIN)[:, None]]
    return a
