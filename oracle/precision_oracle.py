"""Reduced-precision and pruned variants of the matching loop -- TEST INFRASTRUCTURE ONLY.

The checker and the study harness of the product's precision tiers (the BF16 and FP8 projections
with an exact re-score at acceptance, the pruned loop); nothing in the product calls this module.  Kilosort's loop
(KS/template_matching.py:141-202, restated in ``ks_oracle.run_matching``) scores every template at
every sample from an exact projection.  Here:

* ``project_rounded``: the projection B = Wall3 . Bpc with both operands rounded to e4m3 / e5m2 /
  bf16 (round to nearest even, per-template scales on Wall3 and per-(component, channel) scales on
  Bpc, each the row's largest magnitude over the format's largest finite value), accumulated
  exactly.  Those activation scales see the whole window (dynamic, non-causal); with ``act_scale``
  they are static instead, as the FP8 kernel runs them: per-(component, channel) scales fixed once
  from a calibration window (``calibrate_act_scale``: twice the row's largest magnitude over the
  format's largest finite value) and folded into the template operand, whose per-template scale
  is then taken after the fold; values beyond the calibrated range saturate;
* ``run_matching_variant``: Kilosort's loop on such scores, optionally re-scoring every accepted
  candidate exactly (exact initial score minus rounded initial score added to the running score;
  candidates whose exact score misses the threshold are dropped from then on), or restricted to
  the ``keep`` templates per sample with the largest initial (rounded) scores, scored exactly.
  ``keep = T`` with exact scores is Kilosort's loop.

``study()`` prints the agreement table quoted in the design notes (384 channels, 500 templates,
8 windows of the seeded generator at 10 and 40 Hz; a few minutes on a CPU).
"""
from __future__ import annotations

import numpy as np

from . import ks_oracle as ko

MAX_FINITE = {"e4m3": 448.0, "e5m2": 57344.0}
MANT_BITS = {"e4m3": 3, "e5m2": 2}
MIN_EXP = {"e4m3": -6, "e5m2": -14}


def round_fp8(x, fmt: str):
    """Round to the nearest e4m3 / e5m2 value (ties to even), saturating at the largest finite."""
    x = np.asarray(x, np.float64)
    a = np.minimum(np.abs(x), MAX_FINITE[fmt])
    e = np.maximum(np.floor(np.log2(np.maximum(a, 1e-300))), MIN_EXP[fmt])
    q = 2.0 ** (e - MANT_BITS[fmt])
    return np.sign(x) * np.minimum(np.round(a / q) * q, MAX_FINITE[fmt])


def round_bf16(x):
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def operands(X, U, W):
    """(U2 [T, K*C], Bpc2 [K*C, Wn]) of the projection B = U2 @ Bpc2 (ks_oracle.project)."""
    T, K, C = U.shape
    Bpc = ko.conv_basis(np.asarray(X, np.float64), np.asarray(W, np.float64))      # [C, K, Wn]
    Bpc2 = np.ascontiguousarray(Bpc.transpose(1, 0, 2)).reshape(K * C, -1)
    return np.asarray(U, np.float64).reshape(T, K * C), Bpc2


def calibrate_act_scale(Bpc2, fmt: str = "e4m3"):
    """Static per-(component, channel) activation scales [K*C, 1] from one calibration window's
    Bpc2: twice each row's largest magnitude over the format's largest finite value (1 for an
    all-zero row), so held-out values up to twice as large fit before saturating."""
    m = np.abs(np.asarray(Bpc2, np.float64)).max(1, keepdims=True)
    return np.where(m > 0, 2.0 * m / MAX_FINITE[fmt], 1.0)


def project_rounded(U2, Bpc2, fmt: str, act_scale=None):
    if fmt == "exact":
        return U2 @ Bpc2
    if fmt == "bf16":
        return round_bf16(U2) @ round_bf16(Bpc2)
    m = MAX_FINITE[fmt]
    if act_scale is not None:
        s = np.asarray(act_scale, np.float64).reshape(-1, 1)
        Uf = U2 * s.T                                            # the scale folded into the templates
        r = np.maximum(np.abs(Uf).max(1, keepdims=True), 1e-300) / m
        return (r * round_fp8(Uf / r, fmt)) @ round_fp8(Bpc2 / s, fmt)
    r = np.maximum(np.abs(U2).max(1, keepdims=True), 1e-300) / m
    s = np.maximum(np.abs(Bpc2).max(1, keepdims=True), 1e-300) / m
    return (r * (round_fp8(U2 / r, fmt) * s.T)) @ round_fp8(Bpc2 / s, fmt)


def run_matching_variant(X, U, W, ctc, Th, fmt="exact", rescore=False, keep=None, max_iters=50, block=1,
                         act_scale=None, keep_wide=None, crowd=0.5):
    """-> (st [S, 2] (sample, template), amps [S]).  See the module docstring.  block > 1: one list
    per block of that many consecutive samples (from sample 0), the keep templates of largest Cq
    maximum over the block's samples, scored at every sample of the block.  act_scale: static
    activation scales (``calibrate_act_scale``) for an FP8 format.  keep_wide (> keep): a crowded
    sample -- its keep-th largest Cq above crowd * Th^2 -- lists keep_wide templates instead of keep
    (the sorter's match_keep_wide / match_keep_crowd)."""
    U = np.asarray(U, np.float64)
    ctc = np.asarray(ctc, np.float64)
    nt = W.shape[1]
    nm = (U ** 2).sum(-1).sum(-1)
    U2, Bpc2 = operands(X, U, W)
    B0e = U2 @ Bpc2
    B0q = project_rounded(U2, Bpc2, fmt, act_scale)
    if keep is not None:
        Cq = np.maximum(B0q, 0) ** 2 / nm[:, None]
        mask = np.zeros(B0e.shape, bool)
        if block > 1:
            nw = Cq.shape[1]
            for w0 in range(0, nw, block):
                bm = Cq[:, w0:w0 + block].max(1)
                top = np.argsort(-bm, kind="stable")[:keep]
                mask[np.ix_(top, np.arange(w0, min(nw, w0 + block)))] = True
        else:
            # the keep largest per sample, ties to the lower template (a stable sort of -Cq)
            order = np.argsort(-Cq, axis=0, kind="stable")
            cols = np.arange(B0e.shape[1])
            mask[order[:keep], cols[None, :]] = True
            if keep_wide is not None and keep_wide > keep:
                crowded = Cq[order[keep - 1], cols] > crowd * Th ** 2
                mask[order[keep:keep_wide][:, crowded], cols[crowded][None, :]] = True
        B, D = np.where(mask, B0e, -1e30), None
    else:
        B, D = B0q.copy(), B0e - B0q
    excl = np.zeros(B.shape, bool)
    trange = np.arange(-nt, nt + 1)
    st_l, amp_l = [], []
    for _ in range(max_iters):
        _, Cfmax, imax, Cmax = ko.scores(np.where(excl, -1e30, B), nm, nt)
        xs = np.nonzero((Cmax > Th ** 2) & (np.abs(Cmax - Cfmax) < 1e-9))[0]
        if len(xs) == 0:
            break
        iY = imax[xs]
        score = B[iY, xs] if (D is None or not rescore) else B[iY, xs] + D[iY, xs]
        if rescore and D is not None:
            ok = np.maximum(score, 0) ** 2 / nm[iY] > Th ** 2
            excl[iY[~ok], xs[~ok]] = True
            xs, iY, score = xs[ok], iY[ok], score[ok]
            if len(xs) == 0:
                continue
        amp = score / nm[iY]
        st_l.append(np.stack([xs, iY], 1))
        amp_l.append(amp)
        for j in range(2):
            ix, iy, a = xs[j::2], iY[j::2], amp[j::2]
            if len(ix):
                B[:, ix[:, None] + trange[None, :]] -= a[None, :, None] * ctc[:, iy, :]
    st = np.concatenate(st_l).astype(np.int64) if st_l else np.zeros((0, 2), np.int64)
    return st, (np.concatenate(amp_l) if amp_l else np.zeros(0))


def study(rates=(10.0, 40.0), windows: int = 8, only=None):
    """Agreement with the exact loop of each variant on the 384-channel / 500-template shape
    (``only``: names of the variants to run; all by default).  The static-scale variants take their
    scales from window ``windows``, held out of the scored windows 0 .. windows-1."""
    import sys
    import tempfile
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "tests"))
    from lss_testutil import agreement
    from livespikesorter_gb300 import synth
    variants = [("bf16", dict(fmt="bf16")), ("bf16 re-scored", dict(fmt="bf16", rescore=True)),
                ("e4m3", dict(fmt="e4m3")), ("e4m3 re-scored", dict(fmt="e4m3", rescore=True)),
                ("e5m2 re-scored", dict(fmt="e5m2", rescore=True))] + \
               [(f"e4m3 top-{k}, exact", dict(fmt="e4m3", keep=k)) for k in (4, 8, 16)] + \
               [("e4m3 static re-scored", dict(fmt="e4m3", rescore=True, static=True)),
                ("e4m3 static top-16", dict(fmt="e4m3", keep=16, static=True))]
    if only is not None:
        variants = [v for v in variants if v[0] in only]
    for rate in rates:
        cfg = synth.SynthConfig(n_chan=384, n_units=500, n_samples=(windows + 2) * 1500 + 300, drift_um=20.0,
                                whiten_batch=3000, whiten_batches=3, seed=5, rate_hz=rate)
        rec = synth.make_recording(cfg)
        d = synth.write_oss_input(synth.build_oss_input(rec), Path(tempfile.mkdtemp()) / "oss_input")
        oss = ko.load_oss_input(d)
        tot = {name: [0.0, 0.0, 0] for name, _ in variants}
        # static scales from a calibration window that is not one of the windows scored
        Xc = ko.preprocess(rec.data[windows * 1500:windows * 1500 + 1622].T, oss)
        act = calibrate_act_scale(operands(Xc, oss.Wall3, oss.wPCA)[1])
        for j in range(windows):
            X = ko.preprocess(rec.data[j * 1500:j * 1500 + 1622].T, oss)
            ref, refa = run_matching_variant(X, oss.Wall3, oss.wPCA, oss.ctc, oss.th_learned)
            for name, kw in variants:
                kw = dict(kw)
                if kw.pop("static", False):
                    kw["act_scale"] = act
                st, am = run_matching_variant(X, oss.Wall3, oss.wPCA, oss.ctc, oss.th_learned, **kw)
                a, ok, _ = agreement(ref[:, 0], ref[:, 1], refa, st[:, 0], st[:, 1], am)
                tot[name][0] += a * len(ref)
                tot[name][1] += ok * a * len(ref)
                tot[name][2] += len(ref)
        for name, (m, ok, n) in tot.items():
            print(f"{rate:4.0f} Hz  {name:20s} spikes agree {m / n:.4f}  amplitudes within 1e-3 {ok / max(m, 1e-9):.4f}"
                  f"  (reference spikes {n})")


if __name__ == "__main__":
    study()
