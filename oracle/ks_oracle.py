"""ORACLE -- test infrastructure, not product code.

A CPU restatement (numpy, float64 by default) of the per-batch sorting path that
LiveSpikeSorter's GPU sorter mirrors: Kilosort 4.0.13 as vendored in the reference under
src/Python/run_online_spikes/Lib/site-packages/kilosort/ (abbreviated ``KS/`` below).
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import this module, and only as the checker; the product path never calls it.

Pinned against the vendored Kilosort code run in the build container (fixtures in
``tests/golden/``, generated by ``tests/golden/make_golden.py``) and against the
reference's only self-contained known-answer case (src/Python/conv1d_test.py).

Functions and the reference lines they restate:

* ``read_npy_cnpy``      -- cnpy's ``npy_load``: header parsed, ``fortran_order`` ignored for
                            the data (External/CNPY/cnpy.cpp:62-73,180-184)
* ``load_oss_input``     -- the sorter's load step (src/SpikeSorter/OnlineSpikesV2.cu:454-638)
* ``padded_batch``       -- ``BinaryRWFile.padded_batch_to_torch`` (KS/io.py:584-637)
* ``preprocess``         -- ``BinaryFiltered.filter`` (KS/io.py:757-790) with ``fft_highpass``
                            (KS/preprocessing.py:138-154)
* ``run_matching``       -- ``run_matching`` (KS/template_matching.py:128-202)
* ``pc_features``        -- the ``xfeat`` lines of ``extract`` (KS/template_matching.py:50-51)
* ``spike_positions``    -- ``compute_spike_positions`` (KS/postprocessing.py:33-46)
* ``stream_times``       -- the spike-time formula of ``extract`` (KS/template_matching.py:56-68)
* ``remove_duplicates``  -- KS/postprocessing.py:9-30
* ``nearest_centroid``   -- ``OnlineSpikesV2::closestCluster`` (OnlineSpikesV2.cu:1058-1074)
* ``sos_highpass`` / ``sort_stream_biquad`` -- the sorter's stateful high-pass mode, which has no
                            counterpart in the reference: Kilosort's filter design
                            (KS/preprocessing.py:121-136, ``butter(3, 300, 'high')``) run forward
                            with ``scipy.signal.sosfilt`` in float64 over the stream, then the median
                            CAR and ``(M @ Wrot)``; the matching after it is Kilosort's
"""
from __future__ import annotations

import dataclasses
from pathlib import Path

import numpy as np
from numpy.lib.stride_tricks import sliding_window_view

# ----------------------------------------------------------------------------------------
# loading (cnpy semantics)
# ----------------------------------------------------------------------------------------


def read_npy_cnpy(path) -> np.ndarray:
    """Read a .npy the way cnpy does: shape and word size from the header, the payload taken
    in file order as a C-ordered array (``fortran_order`` is parsed but not applied)."""
    with open(path, "rb") as f:
        version = np.lib.format.read_magic(f)
        if version == (1, 0):
            shape, _fortran, dtype = np.lib.format.read_array_header_1_0(f)
        else:
            shape, _fortran, dtype = np.lib.format.read_array_header_2_0(f)
        count = int(np.prod(shape)) if len(shape) else 1
        data = np.fromfile(f, dtype=dtype, count=count)
    return data.reshape(shape)


@dataclasses.dataclass
class OssArrays:
    Wall3: np.ndarray
    ctc: np.ndarray
    wPCA: np.ndarray
    pre_wf: np.ndarray
    whitening: np.ndarray
    drift: np.ndarray
    iCC: np.ndarray
    iU: np.ndarray
    Ucc: np.ndarray
    hp_filter: np.ndarray
    xc: np.ndarray
    yc: np.ndarray
    centroids: np.ndarray
    nt0min: int
    n_nearest: int
    th_learned: float
    dup_bins: int
    n_final: int


def oss_from_arrays(z) -> OssArrays:
    """OssArrays from a mapping holding the exported arrays plus ``misc`` =
    [nt0min, numNearestChans, Th_learned, duplicate_spike_bins] (the golden fixtures)."""
    misc = np.asarray(z["misc"])
    cent = np.asarray(z["centroids"]).astype(np.float64).reshape(-1, 2)
    return OssArrays(
        Wall3=z["Wall3"], ctc=z["ctc"], wPCA=z["wPCA"], pre_wf=z["pre_wf"], whitening=z["whitening"],
        drift=z["drift"], iCC=z["iCC"], iU=z["iU"], Ucc=z["Ucc"], hp_filter=z["hp_filter"],
        xc=z["xc"], yc=z["yc"], centroids=cent, nt0min=int(misc[0]), n_nearest=int(misc[1]),
        th_learned=float(misc[2]), dup_bins=int(misc[3]), n_final=len(cent))


def load_oss_input(d) -> OssArrays:
    d = Path(d)
    rd = lambda n: read_npy_cnpy(d / n)
    misc = {}
    for line in open(d / "misc.txt"):
        if ":" in line:
            k, v = line.strip().split(":", 1)
            misc[k] = v
    templates = rd("templates.npy")
    cent = rd("cluster_centroids.npy").astype(np.float64).reshape(-1, 2)
    return OssArrays(
        Wall3=rd("Wall3.npy"), ctc=rd("ctc.npy"), wPCA=rd("wPCA.npy"),
        pre_wf=rd("preclustered_template_waveforms.npy"), whitening=rd("whiteningMat.npy"),
        drift=rd("drift_matrix.npy"), iCC=rd("iCC.npy"), iU=rd("iU.npy"), Ucc=rd("Ucc.npy"),
        hp_filter=rd("hp_filter.npy"), xc=rd("xc.npy"), yc=rd("yc.npy"), centroids=cent,
        nt0min=int(float(misc["nt0min"])), n_nearest=int(float(misc["numNearestChans"])),
        th_learned=float(misc["Th_learned"]), dup_bins=int(float(misc["duplicate_spike_bins"])),
        n_final=int(templates.shape[0]))


# ----------------------------------------------------------------------------------------
# framing
# ----------------------------------------------------------------------------------------


def n_batches(n_samples: int, NT: int) -> int:
    return int(np.ceil(n_samples / NT))


def padded_batch(data_NC: np.ndarray, ibatch: int, NT: int, nt: int) -> np.ndarray:
    """[C, NT+2nt] float window of batch ``ibatch`` with Kilosort's edge handling (KS/io.py:584-637):
    the first batch replicates its first sample into the left pad, the last batch replicates
    its last sample to the right."""
    N = data_NC.shape[0]
    nb = n_batches(N, NT)
    if ibatch == 0:
        bstart, bend = 0, min(N, NT + nt)
    else:
        bstart = ibatch * NT - nt
        bend = min(N, bstart + NT + 2 * nt)
    d = data_NC[bstart:bend].T.astype(np.float64)
    nsamp = d.shape[1]
    X = np.zeros((data_NC.shape[1], NT + 2 * nt))
    if ibatch == 0:
        X[:, nt:nt + nsamp] = d
        X[:, :nt] = X[:, nt:nt + 1]
    elif ibatch == nb - 1:
        X[:, :nsamp] = d
        X[:, nsamp:] = X[:, nsamp - 1:nsamp]
    else:
        X[:] = d
    return X


# ----------------------------------------------------------------------------------------
# preprocessing
# ----------------------------------------------------------------------------------------


def fft_highpass_kernel(hp_filter: np.ndarray, NT: int) -> np.ndarray:
    """KS/preprocessing.py:138-154: pad with zeros or crop the centred filter to NT."""
    ft = hp_filter.shape[0]
    if ft < NT:
        pad = (NT - ft) // 2
        return np.concatenate([np.zeros(pad), hp_filter, np.zeros(pad + (NT - pad * 2 - ft))])
    if ft > NT:
        crop = (ft - NT) // 2
        return hp_filter[crop:crop + NT]
    return hp_filter


def lower_median(X: np.ndarray, axis: int = 0) -> np.ndarray:
    """torch.median semantics: for an even count, the lower of the two middle values."""
    n = X.shape[axis]
    return np.partition(X, (n - 1) // 2, axis=axis).take((n - 1) // 2, axis=axis)


def preprocess(X: np.ndarray, oss: OssArrays, dtype=np.float64) -> np.ndarray:
    """KS/io.py:757-790 on one [C, W] window: per-channel mean removal, median CAR across
    channels, zero-phase high-pass as a circular correlation with the cropped filter followed
    by ``fftshift``, then ``(M @ Wrot) @ X``."""
    X = X.astype(dtype)
    X = X - X.mean(1, keepdims=True)
    X = X - lower_median(X, 0)[None, :]
    W = X.shape[1]
    h = fft_highpass_kernel(oss.hp_filter.astype(np.float64), W)
    Y = np.real(np.fft.ifft(np.fft.fft(X, axis=-1) * np.conj(np.fft.fft(h)), axis=-1))
    X = np.fft.fftshift(Y, axes=-1).astype(dtype)
    WD = oss.drift.astype(np.float64) @ oss.whitening.astype(np.float64)
    return (WD.astype(dtype) @ X).astype(dtype)


# ----------------------------------------------------------------------------------------
# matching pursuit
# ----------------------------------------------------------------------------------------


def project(X: np.ndarray, U: np.ndarray, W: np.ndarray) -> np.ndarray:
    """B[t, w] = sum_{k,c} U[t,k,c] sum_m X[c, w+m-nt//2] W[k,m]  (KS/template_matching.py:145-146:
    ``conv1d(X, W, padding=nt//2)`` then ``einsum('ijk, kjl -> il')``)."""
    C, Wn = X.shape
    K, nt = W.shape
    Xp = np.pad(X, ((0, 0), (nt // 2, nt // 2)))
    win = sliding_window_view(Xp, nt, axis=1)[:, :Wn, :]          # [C, Wn, nt]
    Bpc = (win.reshape(C * Wn, nt) @ W.T).reshape(C, Wn, K)      # [C, Wn, K]
    Bpc = np.ascontiguousarray(Bpc.transpose(2, 0, 1)).reshape(K * C, Wn)
    return U.reshape(U.shape[0], K * C) @ Bpc


def _maxpool_same(v: np.ndarray, half: int) -> np.ndarray:
    """max_pool1d(kernel 2*half+1, stride 1, padding half): implicit -inf padding."""
    vp = np.concatenate([np.full(half, -np.inf), v, np.full(half, -np.inf)])
    return sliding_window_view(vp, 2 * half + 1).max(1)


def conv_basis(X: np.ndarray, W: np.ndarray) -> np.ndarray:
    """Bpc[c, k, w] = sum_m X[c, w+m-nt//2] W[k, m]: ``conv1d(X, W, padding=nt//2)``."""
    C, Wn = X.shape
    K, nt = W.shape
    Xp = np.pad(X, ((0, 0), (nt // 2, nt // 2)))
    win = sliding_window_view(Xp, nt, axis=1)[:, :Wn, :]
    return np.ascontiguousarray((win @ W.T).transpose(0, 2, 1))


def scores(B: np.ndarray, nm: np.ndarray, nt: int):
    """One scoring pass of the loop (KS/template_matching.py:159-168): returns
    ``Cf, Cfmax, imax, Cmax``."""
    Cf = np.maximum(B, 0) ** 2 / nm[:, None]
    Cf[:, :nt] = 0
    Cf[:, -nt:] = 0
    imax = np.argmax(Cf, 0)
    Cfmax = Cf[imax, np.arange(B.shape[1])]
    return Cf, Cfmax, imax, _maxpool_same(Cfmax, nt)


@dataclasses.dataclass
class MatchResult:
    st: np.ndarray        # [S, 2] int64 (sample in window, template)
    amps: np.ndarray      # [S] amplitude
    Xres: np.ndarray      # [C, W] residual after subtracting every accepted spike
    B0: np.ndarray        # [T, W] projection before the loop
    iters: int            # loop iterations that accepted spikes
    iter_of: np.ndarray   # [S] iteration each spike was accepted in


def run_matching(X: np.ndarray, U: np.ndarray, W: np.ndarray, ctc: np.ndarray, Th: float,
                 max_iters: int = 100, dtype=np.float64, amp_dtype=None) -> MatchResult:
    """KS/template_matching.py:128-202.

    Per iteration: ``Cf = relu(B)^2 / nm`` with the first and last nt samples zeroed; the
    per-sample max over templates; a (2nt+1) max pool; accept samples where the pooled
    value exceeds ``Th^2`` and equals the per-sample max (|diff| < 1e-9); amplitude
    ``B[iY, iX] / nm[iY]``; then subtract every accepted spike from ``Xres`` (waveform
    ``U[iY] @ W`` over nt samples) and from ``B`` (``ctc[:, iY, :]`` over 2nt+1 samples) in
    two interleaved passes (``j::2``), where index assignment does not accumulate repeated
    indices -- the reference's own semantics.  ``amp_dtype`` rounds the stored amplitudes
    (the reference's buffer is float32, line 151); ``None`` keeps ``dtype``.
    """
    U = U.astype(dtype)
    W = W.astype(dtype)
    ctc = ctc.astype(dtype)
    X = X.astype(dtype)
    nt = W.shape[1]
    Th = float(Th)
    nm = (U ** 2).sum(-1).sum(-1)
    B = project(X, U, W).astype(dtype)
    B0 = B.copy()
    trange = np.arange(-nt, nt + 1)
    tiwave = np.arange(-(nt // 2), nt // 2 + 1)
    st_l, amp_l, it_l = [], [], []
    Xres = X.copy()
    iters = 0
    for it in range(max_iters):
        _, Cfmax, imax, Cmax = scores(B, nm, nt)
        xs = np.nonzero((Cmax > Th ** 2) & (np.abs(Cmax - Cfmax) < 1e-9))[0]
        if len(xs) == 0:
            break
        iters += 1
        iY = imax[xs]
        amp = B[iY, xs] / nm[iY]
        if amp_dtype is not None:
            amp = amp.astype(amp_dtype).astype(dtype)
        st_l.append(np.stack([xs, iY], 1))
        amp_l.append(amp)
        it_l.append(np.full(len(xs), it))
        for j in range(2):
            ix, iy, a = xs[j::2], iY[j::2], amp[j::2]
            if len(ix) == 0:
                continue
            wf = np.einsum("ijk,jl->kil", U[iy], W)                      # [C, n, nt]
            Xres[:, ix[:, None] + tiwave[None, :]] -= a[None, :, None] * wf
            B[:, ix[:, None] + trange[None, :]] -= a[None, :, None] * ctc[:, iy, :]
    st = np.concatenate(st_l).astype(np.int64) if st_l else np.zeros((0, 2), np.int64)
    amps = np.concatenate(amp_l) if amp_l else np.zeros(0, dtype)
    iter_of = np.concatenate(it_l) if it_l else np.zeros(0, np.int64)
    return MatchResult(st=st, amps=amps, Xres=Xres, B0=B0, iters=iters, iter_of=iter_of)


def pc_features(Xres: np.ndarray, st: np.ndarray, amps: np.ndarray, oss: OssArrays,
                dtype=np.float64) -> np.ndarray:
    """tF [S, nC, K]:  Xres[iCC[:, iU[t]], s + tiwave] @ wPCA.T + amp * Ucc[:, t]
    (KS/template_matching.py:50-51, transposed as at line 73)."""
    W = oss.wPCA.astype(dtype)
    nt = W.shape[1]
    if len(st) == 0:
        return np.zeros((0, oss.iCC.shape[0], W.shape[0]), dtype)
    tiwave = np.arange(-(nt // 2), nt // 2 + 1)
    chans = oss.iCC[:, oss.iU[st[:, 1]]]                         # [nC, S]
    times = st[:, 0][:, None] + tiwave[None, :]                   # [S, nt]
    seg = Xres[chans[:, :, None], times[None, :, :]]              # [nC, S, nt]
    xfeat = seg @ W.T                                             # [nC, S, K]
    xfeat = xfeat + amps[None, :, None] * oss.Ucc[:, st[:, 1]].astype(dtype)
    return np.ascontiguousarray(xfeat.transpose(1, 0, 2))


def spike_positions(tF: np.ndarray, st: np.ndarray, oss: OssArrays):
    """KS/postprocessing.py:33-46: feature-energy weighted mean of the nearest sites."""
    if len(st) == 0:
        return np.zeros(0), np.zeros(0)
    tmass = (tF ** 2).sum(-1)
    tmass = tmass / tmass.sum(1, keepdims=True)
    chs = oss.iCC[:, oss.iU[st[:, 1]]]
    xs = (oss.xc.astype(np.float64)[chs.T] * tmass).sum(1)
    ys = (oss.yc.astype(np.float64)[chs.T] * tmass).sum(1)
    return xs, ys


# ----------------------------------------------------------------------------------------
# egress
# ----------------------------------------------------------------------------------------


def stream_times(s_in_window: np.ndarray, window_start: int, nt: int, nt0min: int) -> np.ndarray:
    """Stream sample of a spike found at window sample s (KS/template_matching.py:68):
    ``(s - nt) + ibatch*NT - nt//2 + nt0min`` where the window starts at ``ibatch*NT - nt``."""
    return window_start + s_in_window - nt // 2 + nt0min


def nearest_centroid(x: np.ndarray, y: np.ndarray, centroids: np.ndarray) -> np.ndarray:
    """Index of the closest final-cluster centroid in (x, y), first one on ties
    (OnlineSpikesV2.cu:1058-1074)."""
    if len(x) == 0:
        return np.zeros(0, np.int64)
    d = (x[:, None] - centroids[None, :, 0]) ** 2 + (y[:, None] - centroids[None, :, 1]) ** 2
    return np.argmin(d, 1).astype(np.int64)


def pc_score_cluster(tF: np.ndarray, xs: np.ndarray, ys: np.ndarray, centroids: np.ndarray,
                     centroids_pca: np.ndarray, radius: float) -> np.ndarray:
    """Final cluster by PC score (OnlineKilosort.py:233-284): among the clusters whose (x, y)
    centroid lies within ``radius`` of the spike, argmax (first on ties) of 2 tF.mu - |mu|^2 with
    tF flattened to [nC*K] and mu a row of ``centroids_pca``; -1 when no centroid is that close."""
    if len(xs) == 0:
        return np.zeros(0, np.int64)
    X = tF.reshape(len(tF), -1).astype(np.float64)
    mu = np.asarray(centroids_pca, np.float64)
    sc = 2.0 * X @ mu.T - (mu ** 2).sum(1)[None, :]
    c = np.asarray(centroids, np.float64)
    d2 = (xs[:, None] - c[None, :, 0]) ** 2 + (ys[:, None] - c[None, :, 1]) ** 2
    near = d2 <= radius ** 2
    best = np.argmax(np.where(near, sc, -np.inf), 1).astype(np.int64)
    best[~near.any(1)] = -1
    return best


def remove_duplicates(times: np.ndarray, clusters: np.ndarray, dt: int, last=None):
    """KS/postprocessing.py:9-30 over time-sorted spikes; ``last`` carries each cluster's last
    kept time across calls (streaming).  Spikes without a cluster (-1) are all kept.  Returns the
    keep mask."""
    last = {} if last is None else last
    keep = np.zeros(len(times), bool)
    for i in range(len(times)):
        t, c = int(times[i]), int(clusters[i])
        if c < 0:
            keep[i] = True
            continue
        t0 = last.get(c, t - dt)
        if t >= t0 + dt:
            last[c] = t
            keep[i] = True
    return keep


# ----------------------------------------------------------------------------------------
# composition
# ----------------------------------------------------------------------------------------


@dataclasses.dataclass
class WindowResult:
    X: np.ndarray         # [C, W] preprocessed window
    match: MatchResult
    tF: np.ndarray        # [S, nC, K]
    xs: np.ndarray
    ys: np.ndarray


def sort_window(window_CW: np.ndarray, oss: OssArrays, max_iters: int = 50,
                dtype=np.float64, amp_dtype=None) -> WindowResult:
    return sort_preprocessed(preprocess(window_CW, oss, dtype=dtype), oss, max_iters, dtype, amp_dtype)


def sort_preprocessed(X: np.ndarray, oss: OssArrays, max_iters: int = 50, dtype=np.float64,
                      amp_dtype=None) -> WindowResult:
    """Kilosort's matching, features and positions on an already preprocessed [C, W] window."""
    m = run_matching(X, oss.Wall3, oss.wPCA, oss.ctc, oss.th_learned, max_iters=max_iters,
                     dtype=dtype, amp_dtype=amp_dtype)
    tF = pc_features(m.Xres, m.st, m.amps, oss, dtype=dtype)
    xs, ys = spike_positions(tF, m.st, oss)
    return WindowResult(X=X, match=m, tF=tF, xs=xs, ys=ys)


def sort_stream(data_NC: np.ndarray, oss: OssArrays, NT: int, max_iters: int = 50,
                dtype=np.float64, batches=None, centroids_pca=None, radius: float = 80.0):
    """Kilosort ``extract`` over a whole recording (KS/template_matching.py:28-85) plus the
    final-cluster assignment (nearest centroid, or the PC-score rule when ``centroids_pca`` is
    given) and duplicate removal.  Returns per-spike arrays sorted by time:
    ``time, template, cluster, amp, x, y, tF`` and the keep mask of the duplicate pass."""
    nt = oss.wPCA.shape[1]
    nb = n_batches(data_NC.shape[0], NT)
    out = {k: [] for k in ("time", "template", "amp", "x", "y", "tF")}
    for ib in (range(nb) if batches is None else batches):
        r = sort_window(padded_batch(data_NC, ib, NT, nt), oss, max_iters=max_iters, dtype=dtype)
        t = stream_times(r.match.st[:, 0], ib * NT - nt, nt, oss.nt0min)
        keep = t >= 0 if ib == 0 else np.ones(len(t), bool)
        out["time"].append(t[keep])
        out["template"].append(r.match.st[keep, 1])
        out["amp"].append(r.match.amps[keep])
        out["x"].append(r.xs[keep])
        out["y"].append(r.ys[keep])
        out["tF"].append(r.tF[keep])
    res = {k: (np.concatenate(v) if len(v) else np.zeros(0)) for k, v in out.items()}
    order = np.lexsort((res["template"], res["time"]))
    res = {k: v[order] for k, v in res.items()}
    if centroids_pca is None:
        res["cluster"] = nearest_centroid(res["x"], res["y"], oss.centroids)
    else:
        res["cluster"] = pc_score_cluster(res["tF"], res["x"], res["y"], oss.centroids, centroids_pca, radius)
    res["keep"] = remove_duplicates(res["time"], res["cluster"], oss.dup_bins)
    return res


# ----------------------------------------------------------------------------------------
# stateful high-pass mode (no counterpart in the reference)
# ----------------------------------------------------------------------------------------


def highpass_sos(order: int = 3, cutoff_hz: float = 300.0, fs: float = 30000.0) -> np.ndarray:
    """Kilosort's high-pass design (KS/preprocessing.py:121-136) as second-order sections."""
    from scipy.signal import butter
    return butter(order, cutoff_hz, btype="high", fs=fs, output="sos")


def sos_highpass(x_NC: np.ndarray, sos: np.ndarray, zi=None):
    """The causal high-pass along time (axis 0) in float64; from the steady state of the first row
    (``sosfilt_zi * x[0]``) unless ``zi`` [n_sections, 2, C] continues an earlier call.  Returns
    the filtered rows and the final state."""
    from scipy.signal import sosfilt, sosfilt_zi
    x = np.asarray(x_NC, np.float64)
    if zi is None:
        zi = sosfilt_zi(sos)[:, :, None] * x[0][None, None, :]
    return sosfilt(sos, x, axis=0, zi=zi)


def biquad_padded_stream(data_NC: np.ndarray, NT: int, nt: int) -> np.ndarray:
    """The rows the streaming sorter filters, with Kilosort's batch framing (KS/io.py:584-637):
    nt copies of the first sample, the recording, then the last window's right pad (copies of the
    last sample, or zeros when the first batch is also the last); window j = rows [j NT, j NT + W)."""
    N, C = data_NC.shape
    nb = n_batches(N, NT)
    W = NT + 2 * nt
    tail = (nb - 1) * NT + W - nt - N
    x = np.asarray(data_NC, np.float64)
    pad = np.zeros((max(tail, 0), C)) if nb == 1 else np.repeat(x[-1:], max(tail, 0), axis=0)
    return np.concatenate([np.repeat(x[:1], nt, axis=0), x, pad])[: (nb - 1) * NT + W]


def preprocess_biquad(F_WC: np.ndarray, oss: OssArrays) -> np.ndarray:
    """Filtered rows [W, C] of one window -> [C, W]: lower-median CAR per sample, then (M @ Wrot)."""
    X = np.asarray(F_WC, np.float64).T
    X = X - lower_median(X, 0)[None, :]
    WD = oss.drift.astype(np.float64) @ oss.whitening.astype(np.float64)
    return WD @ X


def sort_stream_biquad(data_NC: np.ndarray, oss: OssArrays, NT: int, sos: np.ndarray, max_iters: int = 50):
    """``sort_stream`` with the stateful high-pass: the padded stream filtered once, forward, each
    batch window cut from it, CAR'd, whitened and matched.  Nearest-centroid clusters and duplicate
    removal as in ``sort_stream``."""
    nt = oss.wPCA.shape[1]
    W = NT + 2 * nt
    F, _ = sos_highpass(biquad_padded_stream(data_NC, NT, nt), sos)
    nb = n_batches(data_NC.shape[0], NT)
    out = {k: [] for k in ("time", "template", "amp", "x", "y", "tF")}
    for ib in range(nb):
        r = sort_preprocessed(preprocess_biquad(F[ib * NT: ib * NT + W], oss), oss, max_iters=max_iters)
        t = stream_times(r.match.st[:, 0], ib * NT - nt, nt, oss.nt0min)
        keep = t >= 0 if ib == 0 else np.ones(len(t), bool)
        out["time"].append(t[keep])
        out["template"].append(r.match.st[keep, 1])
        out["amp"].append(r.match.amps[keep])
        out["x"].append(r.xs[keep])
        out["y"].append(r.ys[keep])
        out["tF"].append(r.tF[keep])
    res = {k: (np.concatenate(v) if len(v) else np.zeros(0)) for k, v in out.items()}
    order = np.lexsort((res["template"], res["time"]))
    res = {k: v[order] for k, v in res.items()}
    res["cluster"] = nearest_centroid(res["x"], res["y"], oss.centroids)
    res["keep"] = remove_duplicates(res["time"], res["cluster"], oss.dup_bins)
    return res
