"""Seeded synthetic Neuropixels-style recordings and their Kilosort4 ``oss_input/`` export.

The sorter is driven by an ``oss_input/`` directory that the reference's offline step
writes from a Kilosort 4.0.13 run (src/Python/run_online_spikes.py:598-672 with
crop_methods.py:158-175).  No recording and no Kilosort output ships with the
reference, so this module builds both from one seed:

* a probe (two columns 32 um apart, 20 um row pitch),
* ``n_units`` units, each a spatial Gaussian (sigma 30 um) around a random site times a
  random mix of ``n_pcs`` orthonormal biphasic temporal bases (the bases are ``wPCA``),
* Poisson spike trains with a refractory period and lognormal amplitudes,
* N(0, noise_std^2) noise, rounded to int16 in ``[samples][channels]`` order (SpikeGLX order),
* an optional rigid drift (a 0..drift_um sinusoid along the shank),

and then the export: the high-pass filter (Kilosort preprocessing.py:121-136), the
local whitening matrix from the data covariance (preprocessing.py:19-35, 96-119), the
drift interpolation matrix (preprocessing.py:44-69, datashift.py:212-219), templates in
whitened PC space (``Wall3``), ``ctc`` (template_matching.py:110-121), ``iCC/iU/Ucc``
(template_matching.py:20-26) and ``misc.txt``.  Every file is written with the dtype
and memory order the reference exporter produces, including the Fortran-ordered
``drift_matrix.npy`` (run_online_spikes.py:628 saves ``M.T``) that cnpy reads back as
``M`` because it ignores ``fortran_order``.
"""
from __future__ import annotations

import dataclasses
import hashlib
import json
import os
from pathlib import Path

import numpy as np

# ----------------------------------------------------------------------------------------
# configuration
# ----------------------------------------------------------------------------------------


@dataclasses.dataclass
class SynthConfig:
    n_chan: int = 96
    n_units: int = 64
    n_samples: int = 60000 + 2 * 61
    fs: float = 30000.0
    nt: int = 61
    n_pcs: int = 6
    nt0min: int = 20
    n_nearest: int = 10
    th_learned: float = 8.0
    duplicate_spike_bins: int = 7
    rate_hz: float = 10.0
    refractory_ms: float = 1.0
    amp_log_mu: float = float(np.log(60.0))
    amp_log_sigma: float = 0.3
    noise_std: float = 10.0
    sig_um: float = 30.0
    pitch_um: float = 20.0
    col_x_um: tuple = (0.0, 32.0)
    drift_um: float = 0.0          # peak-to-peak of the rigid drift sinusoid
    drift_period_s: float = 20.0
    overlap_frac: float = 0.0      # fraction of spikes forced to overlap a spike of a neighbour unit
    whiten_batches: int = 8        # batches used for the covariance estimate
    whiten_batch: int = 4000
    seed: int = 0

    def to_json(self) -> str:
        return json.dumps(dataclasses.asdict(self), sort_keys=True)


def config_small(seed: int = 0) -> SynthConfig:
    """96 channels, 64 units, one 60000-sample batch (+2*nt padding): the CPU-runnable case."""
    return SynthConfig(n_chan=96, n_units=64, n_samples=60000 + 2 * 61, seed=seed)


def config_stream(seconds: float = 60.0, seed: int = 1) -> SynthConfig:
    """384 channels, 500 templates, a streamed recording with a 0-20 um rigid drift."""
    return SynthConfig(n_chan=384, n_units=500, n_samples=int(seconds * 30000), drift_um=20.0, seed=seed)


# ----------------------------------------------------------------------------------------
# geometry, temporal basis, filters
# ----------------------------------------------------------------------------------------


def probe_geometry(n_chan: int, pitch_um: float = 20.0, col_x_um=(0.0, 32.0)):
    """Two-column probe: channel i sits in column i%2 at depth pitch*(i//2)."""
    xc = np.array([col_x_um[i % 2] for i in range(n_chan)], dtype=np.float32)
    yc = (np.arange(n_chan) // 2 * pitch_um).astype(np.float32)
    return xc, yc


def temporal_basis(nt: int, n_pcs: int, nt0min: int) -> np.ndarray:
    """``n_pcs`` orthonormal biphasic bases of length ``nt`` aligned on sample ``nt0min``.

    Gaussian derivatives of two widths around ``nt0min``, orthonormalised in order (QR),
    so the first basis is the dominant biphasic trough/peak shape.  Rows are orthonormal,
    like Kilosort's ``wPCA`` [n_pcs, nt].
    """
    t = np.arange(nt, dtype=np.float64) - nt0min
    cols = []
    for order in range(3):
        for width in (2.5, 5.0):
            g = np.exp(-0.5 * (t / width) ** 2)
            h = [g, -t / width ** 2 * g, (t ** 2 / width ** 4 - 1.0 / width ** 2) * g][order]
            # a slow after-hyperpolarisation so every basis is biphasic
            h = h - 0.25 * np.roll(g, int(2 * width)) * (order == 0)
            cols.append(h)
    A = np.stack(cols[:max(n_pcs, 1)], 1)
    while A.shape[1] < n_pcs:
        A = np.concatenate([A, np.sin(np.pi * (A.shape[1] + 1) * (t - t.min()) / nt)[:, None]], 1)
    Q, R = np.linalg.qr(A[:, :n_pcs])
    Q = Q * np.sign(np.diag(R))[None, :]
    return np.ascontiguousarray(Q.T.astype(np.float32))


def highpass_impulse(fs: float = 30000.0, cutoff: float = 300.0, NT: int = 30122) -> np.ndarray:
    """Zero-phase impulse response of a 3rd-order Butterworth high-pass (filtfilt), float32.

    Restates Kilosort preprocessing.py:121-136 (``get_highpass_filter``): a unit impulse at
    NT//2 pushed through ``filtfilt(butter(3, cutoff, 'high'))``.
    """
    from scipy.signal import butter, filtfilt
    b, a = butter(3, cutoff, fs=fs, btype="high")
    x = np.zeros(NT)
    x[NT // 2] = 1.0
    return filtfilt(b, a, x).astype(np.float32)


def fft_highpass_kernel(hp_filter: np.ndarray, NT: int) -> np.ndarray:
    """Pad or crop the filter to length NT exactly as Kilosort preprocessing.py:138-154."""
    ft = hp_filter.shape[0]
    if ft < NT:
        pad = (NT - ft) // 2
        return np.concatenate([np.zeros(pad, hp_filter.dtype), hp_filter,
                               np.zeros(pad + (NT - pad * 2 - ft), hp_filter.dtype)])
    if ft > NT:
        crop = (ft - NT) // 2
        return hp_filter[crop:crop + NT]
    return hp_filter


def circular_highpass(X: np.ndarray, hp_filter: np.ndarray) -> np.ndarray:
    """fftshift(real(ifft(fft(X) * conj(fft(h))))) along the last axis (Kilosort io.py:771-774)."""
    NT = X.shape[-1]
    h = fft_highpass_kernel(hp_filter.astype(np.float64), NT)
    Y = np.real(np.fft.ifft(np.fft.fft(X, axis=-1) * np.conj(np.fft.fft(h)), axis=-1))
    return np.fft.fftshift(Y, axes=-1)


def kernel2d(xp: np.ndarray, yp: np.ndarray, sig: float) -> np.ndarray:
    ds = ((xp[:, None, :] - yp[None, :, :]) ** 2).sum(-1)
    return np.exp(-ds / (2 * sig ** 2))


def drift_matrix(xc, yc, dshift: float, sig_interp: float = 20.0) -> np.ndarray:
    """Rigid-drift interpolation matrix M (Kilosort preprocessing.py:44-69, nblocks=1),
    with ``iKxx = inv(Kxx + 0.01 I)`` (datashift.py:212-219).  Applied as ``X <- M @ X``."""
    xp = np.stack([xc, yc], 1).astype(np.float64)
    Kxx = kernel2d(xp, xp, sig_interp)
    iKxx = np.linalg.inv(Kxx + 0.01 * np.eye(len(xc)))
    yp = xp.copy()
    yp[:, 1] -= dshift
    Kyx = kernel2d(yp, xp, sig_interp)
    return Kyx @ iKxx


def whitening_local(CC: np.ndarray, xc, yc, nrange: int = 32) -> np.ndarray:
    """Per-channel ZCA whitening over the ``nrange`` nearest sites (Kilosort preprocessing.py:8-35)."""
    n = CC.shape[0]
    Wrot = np.zeros((n, n))
    for j in range(n):
        ds = (xc[j] - xc) ** 2 + (yc[j] - yc) ** 2
        ix = np.argsort(ds)[:nrange]
        E, D, _ = np.linalg.svd(CC[np.ix_(ix, ix)])
        wrot = (E / (D + 1e-6) ** 0.5) @ E.T
        Wrot[j, ix] = wrot[0]
    return Wrot


# ----------------------------------------------------------------------------------------
# units, spike trains, rendering
# ----------------------------------------------------------------------------------------


@dataclasses.dataclass
class Units:
    x0: np.ndarray        # [U] um
    y0: np.ndarray        # [U] um
    coef: np.ndarray      # [U, K] mix of the temporal bases
    wave: np.ndarray      # [U, nt] temporal waveform, peak |.| = 1


@dataclasses.dataclass
class SpikeTrain:
    times: np.ndarray     # [S] int64 sample of alignment (waveform sample nt0min sits here)
    units: np.ndarray     # [S] int64
    amps: np.ndarray      # [S] float32


@dataclasses.dataclass
class Recording:
    cfg: SynthConfig
    data: np.ndarray      # [N, C] int16
    xc: np.ndarray
    yc: np.ndarray
    wPCA: np.ndarray      # [K, nt]
    units: Units
    train: SpikeTrain

    def drift_at(self, sample) -> np.ndarray:
        return drift_um_at(self.cfg, sample)


def drift_um_at(cfg: SynthConfig, sample) -> np.ndarray:
    t = np.asarray(sample, dtype=np.float64) / cfg.fs
    return 0.5 * cfg.drift_um * (1.0 - np.cos(2 * np.pi * t / cfg.drift_period_s))


def make_units(cfg: SynthConfig, wPCA: np.ndarray, xc, yc, rng) -> Units:
    U = cfg.n_units
    x0 = rng.uniform(xc.min(), xc.max(), U)
    y0 = rng.uniform(yc.min() + 10.0, yc.max() - 10.0, U)
    coef = rng.normal(0.0, 1.0, (U, cfg.n_pcs))
    coef[:, 0] = np.abs(coef[:, 0]) * 2.0 + 2.0     # dominant biphasic component
    wave = coef @ wPCA.astype(np.float64)
    wave /= np.abs(wave).max(1, keepdims=True)
    return Units(x0=x0, y0=y0, coef=coef, wave=wave.astype(np.float64))


def make_spike_train(cfg: SynthConfig, rng) -> SpikeTrain:
    ref = cfg.refractory_ms * 1e-3
    rate_eff = 1.0 / max(1.0 / cfg.rate_hz - ref, 1e-6)
    dur = cfg.n_samples / cfg.fs
    lo, hi = cfg.nt, cfg.n_samples - cfg.nt       # keep whole waveforms inside the recording
    times, units = [], []
    for u in range(cfg.n_units):
        n_exp = int(dur * cfg.rate_hz * 1.5) + 10
        isi = ref + rng.exponential(1.0 / rate_eff, n_exp)
        t = np.cumsum(isi) + rng.uniform(0, 1.0 / cfg.rate_hz)
        t = np.round(t[t < dur] * cfg.fs).astype(np.int64)
        t = t[(t >= lo) & (t < hi)]
        times.append(t)
        units.append(np.full(t.shape, u, np.int64))
    times = np.concatenate(times) if times else np.zeros(0, np.int64)
    units = np.concatenate(units) if units else np.zeros(0, np.int64)
    if cfg.overlap_frac > 0 and len(times):
        # move a fraction of spikes to within 1 ms of a spike of another unit
        n_move = int(cfg.overlap_frac * len(times))
        idx = rng.choice(len(times), n_move, replace=False)
        partners = rng.integers(0, len(times), n_move)
        jitter = rng.integers(-int(cfg.fs * 1e-3), int(cfg.fs * 1e-3) + 1, n_move)
        times[idx] = np.clip(times[partners] + jitter, lo, hi - 1)
    amps = np.exp(rng.normal(cfg.amp_log_mu, cfg.amp_log_sigma, len(times))).astype(np.float32)
    order = np.argsort(times, kind="stable")
    return SpikeTrain(times=times[order], units=units[order], amps=amps[order])


def spatial_footprint(cfg: SynthConfig, units: Units, xc, yc, dy: float) -> np.ndarray:
    """[U, C] Gaussian footprints with the units displaced by ``dy`` um along the shank."""
    d2 = (xc[None, :] - units.x0[:, None]) ** 2 + (yc[None, :] - (units.y0[:, None] + dy)) ** 2
    return np.exp(-d2 / (2 * cfg.sig_um ** 2))


def render(cfg: SynthConfig, units: Units, train: SpikeTrain, xc, yc, rng, chunk: int = 1500) -> np.ndarray:
    """int16 [N, C] = round(noise + sum_spikes amp * wave[unit] (x) footprint[unit](drift))."""
    N, C, nt = cfg.n_samples, cfg.n_chan, cfg.nt
    out = np.empty((N, C), np.int16)
    starts = train.times - cfg.nt0min            # first waveform sample of each spike
    m = np.arange(nt)
    for n0 in range(0, N, chunk):
        n1 = min(N, n0 + chunk)
        x = rng.standard_normal((n1 - n0, C), dtype=np.float32) * np.float32(cfg.noise_std)
        sel = np.nonzero((starts < n1) & (starts + nt > n0))[0]
        if len(sel):
            pos = starts[sel, None] + m[None, :]                     # [s, nt]
            val = train.amps[sel, None] * units.wave[train.units[sel]]   # [s, nt]
            inside = (pos >= n0) & (pos < n1)
            sig = np.zeros((n1 - n0, cfg.n_units))
            np.add.at(sig, (pos[inside] - n0, np.broadcast_to(train.units[sel, None], pos.shape)[inside]),
                      val[inside])
            S = spatial_footprint(cfg, units, xc, yc, float(drift_um_at(cfg, 0.5 * (n0 + n1))))
            x += (sig @ S).astype(np.float32)
        out[n0:n1] = np.clip(np.rint(x), -32768, 32767).astype(np.int16)
    return out


def make_recording(cfg: SynthConfig) -> Recording:
    rng = np.random.default_rng(cfg.seed)
    xc, yc = probe_geometry(cfg.n_chan, cfg.pitch_um, cfg.col_x_um)
    wPCA = temporal_basis(cfg.nt, cfg.n_pcs, cfg.nt0min)
    units = make_units(cfg, wPCA, xc, yc, rng)
    train = make_spike_train(cfg, rng)
    data = render(cfg, units, train, xc, yc, rng)
    return Recording(cfg=cfg, data=data, xc=xc, yc=yc, wPCA=wPCA, units=units, train=train)


def rerecord(rec: Recording, seed: int, rate_hz: float = None, n_samples: int = None) -> Recording:
    """A new recording of the same units and probe (so the same oss_input/ applies): fresh spike
    times, amplitudes and noise from ``seed``, optionally another firing rate and length."""
    cfg = dataclasses.replace(rec.cfg, seed=seed, rate_hz=rate_hz if rate_hz is not None else rec.cfg.rate_hz,
                              n_samples=n_samples if n_samples is not None else rec.cfg.n_samples)
    rng = np.random.default_rng(seed)
    train = make_spike_train(cfg, rng)
    data = render(cfg, rec.units, train, rec.xc, rec.yc, rng)
    return Recording(cfg=cfg, data=data, xc=rec.xc, yc=rec.yc, wPCA=rec.wPCA, units=rec.units, train=train)


# ----------------------------------------------------------------------------------------
# export: the oss_input/ directory
# ----------------------------------------------------------------------------------------


def _car_highpass(Xw: np.ndarray, hp: np.ndarray) -> np.ndarray:
    """Mean removal, median CAR and the circular high-pass on one [C, W] window (float64)."""
    X = Xw - Xw.mean(1, keepdims=True)
    Cn = X.shape[0]
    med = np.sort(X, 0)[(Cn - 1) // 2]
    X = X - med[None, :]
    return circular_highpass(X, hp)


def covariance(rec: Recording, hp: np.ndarray) -> np.ndarray:
    """Channel covariance of preprocessed batches (Kilosort preprocessing.py:96-119)."""
    cfg = rec.cfg
    NT, nt = cfg.whiten_batch, cfg.nt
    n_b = max(1, min(cfg.whiten_batches, (cfg.n_samples - 2 * nt) // NT))
    CC = np.zeros((cfg.n_chan, cfg.n_chan))
    for j in range(n_b):
        w = rec.data[j * NT: j * NT + NT + 2 * nt].T.astype(np.float64)
        X = _car_highpass(w, hp)[:, nt:-nt]
        CC += X @ X.T / X.shape[1]
    return CC / n_b


def prepare_matching(wPCA: np.ndarray, U: np.ndarray) -> np.ndarray:
    """ctc[i, j, l] = sum_{k,m} (U_i . U_j)[k, m] WtW[k, m, l]  (Kilosort template_matching.py:110-121).

    ``WtW[k, m, :]`` is the full cross-correlation of basis rows k and m (length 2nt+1),
    flipped as in the reference, computed in float64 and returned as float32.
    """
    K, nt = wPCA.shape
    W = wPCA.astype(np.float64)
    WtW = np.zeros((K, K, 2 * nt + 1))
    for k in range(K):
        for m in range(K):
            # torch conv1d(W_k, W_m, padding=nt) is a cross-correlation: out[s] = sum_j Wk[j+s-nt] Wm[j]
            full = np.correlate(np.pad(W[k], (nt, nt)), W[m], mode="valid")  # length 2nt+1
            WtW[k, m] = full[::-1]
    U64 = U.astype(np.float64)
    UtU = np.einsum("ikl,jml->ijkm", U64, U64, optimize=True)
    ctc = np.einsum("ijkm,kml->ijl", UtU, WtW, optimize=True)
    return ctc.astype(np.float32)


def prepare_extract(xc, yc, U: np.ndarray, nC: int):
    """iCC [nC, C] nearest-site lists, iU [T] peak channel, Ucc [nC, T, K]
    (Kilosort template_matching.py:20-26)."""
    ds = (xc - xc[:, None]) ** 2 + (yc - yc[:, None]) ** 2
    iCC = np.argsort(ds, 0)[:nC].astype(np.int64)
    iU = np.argmax((U.astype(np.float64) ** 2).sum(1), -1).astype(np.int64)
    T = U.shape[0]
    Ucc = U[np.arange(T)[None, :], :, iCC[:, iU]]           # [nC, T, K]
    return iCC, iU, np.ascontiguousarray(Ucc.astype(np.float32))


def processed_templates(rec: Recording, hp: np.ndarray, WD: np.ndarray, dy: float) -> np.ndarray:
    """Wall3 [U, K, C]: each unit's waveform pushed through high-pass and ``WD = M @ Wrot``,
    then projected on the temporal basis over the nt-sample window it occupies."""
    cfg = rec.cfg
    nt, pad = cfg.nt, 1024
    S = spatial_footprint(cfg, rec.units, rec.xc, rec.yc, dy)        # [U, C]
    L = nt + 2 * pad
    h = fft_highpass_kernel(hp.astype(np.float64), L)
    Hf = np.conj(np.fft.fft(h))
    wave = np.zeros((cfg.n_units, L))
    wave[:, pad:pad + nt] = rec.units.wave
    filt = np.fft.fftshift(np.real(np.fft.ifft(np.fft.fft(wave, axis=-1) * Hf, axis=-1)), axes=-1)
    seg = filt[:, pad:pad + nt]                                      # [U, nt]
    coefs = seg @ rec.wPCA.astype(np.float64).T                      # [U, K]
    # a rank-1 (space x time) unit: Wall3[u, k, :] = coef[u, k] * (WD @ footprint[u])
    spat = S @ WD.T                                                  # [U, C]
    Wall3 = coefs[:, :, None] * spat[:, None, :]
    return Wall3.astype(np.float32)


@dataclasses.dataclass
class OssInput:
    """The in-memory content of one oss_input/ directory (the sorter's load contract)."""
    templates: np.ndarray          # [T, M, C] f32
    Wall3: np.ndarray              # [Tu, K, C] f32
    ctc: np.ndarray                # [Tu, Tu, 2M+1] f32
    wPCA: np.ndarray               # [K, M] f32
    pre_wf: np.ndarray             # [Tu, M, C] f32
    whitening: np.ndarray          # [C, C] f32   (applied as X <- Wrot @ X)
    drift: np.ndarray              # [C, C] f32   (applied as X <- M @ X)
    iCC: np.ndarray                # [nC, C] i64
    iU: np.ndarray                 # [Tu] i64
    Ucc: np.ndarray                # [nC, Tu, K] f32
    hp_filter: np.ndarray          # [30122] f32
    xc: np.ndarray
    yc: np.ndarray
    channel_map: np.ndarray        # [C] i32
    template_map: np.ndarray       # [T] i32
    centroids: np.ndarray          # [T, 2] f32 final-cluster (x, y)
    centroids_pca: np.ndarray      # [T, K] f32
    spike_templates: np.ndarray    # [S] i64
    misc: dict


def build_oss_input(rec: Recording) -> OssInput:
    cfg = rec.cfg
    hp = highpass_impulse(cfg.fs)
    CC = covariance(rec, hp)
    Wrot = whitening_local(CC, rec.xc.astype(np.float64), rec.yc.astype(np.float64))
    d_last = float(drift_um_at(cfg, cfg.n_samples - 1))
    M = drift_matrix(rec.xc, rec.yc, d_last)
    WD = M @ Wrot
    Wall3 = processed_templates(rec, hp, WD, d_last)
    ctc = prepare_matching(rec.wPCA, Wall3)
    iCC, iU, Ucc = prepare_extract(rec.xc.astype(np.float64), rec.yc.astype(np.float64), Wall3, cfg.n_nearest)
    pre_wf = np.einsum("ijk,jl->ilk", Wall3.astype(np.float64), rec.wPCA.astype(np.float64)).astype(np.float32)
    T = cfg.n_units
    centroids = np.stack([rec.units.x0, rec.units.y0], 1).astype(np.float32)
    centroids_pca = Wall3[np.arange(T), :, iU].astype(np.float32)
    n_keep = min(len(rec.train.units), 100000)
    misc = {"nt0min": cfg.nt0min, "numNearestChans": cfg.n_nearest,
            "Th_learned": cfg.th_learned, "duplicate_spike_bins": cfg.duplicate_spike_bins}
    return OssInput(templates=pre_wf.copy(), Wall3=Wall3, ctc=ctc, wPCA=rec.wPCA.astype(np.float32),
                    pre_wf=pre_wf, whitening=Wrot.astype(np.float32), drift=M.astype(np.float32),
                    iCC=iCC, iU=iU, Ucc=Ucc, hp_filter=hp, xc=rec.xc, yc=rec.yc,
                    channel_map=np.arange(cfg.n_chan, dtype=np.int32),
                    template_map=np.arange(T, dtype=np.int32), centroids=centroids,
                    centroids_pca=centroids_pca, spike_templates=rec.train.units[:n_keep].copy(), misc=misc)


def centroids_pca_flat(oss: OssInput) -> np.ndarray:
    """[T_final, nC*K] centroid features of the PC-score cluster rule: each final cluster's
    template PC features on its template's nearest channels, flattened channel-major (the
    layout OnlineKilosort.py:211-230 builds from Wall and pc_feature_ind).  Here the final
    clusters are the units, so their templates are the rows of Wall3."""
    T = oss.Wall3.shape[0]
    chans = oss.iCC[:, oss.iU]                                   # [nC, T]
    return np.stack([oss.Wall3[t][:, chans[:, t]].T.reshape(-1) for t in range(T)]).astype(np.float32)


def write_oss_input(oss: OssInput, out_dir) -> Path:
    """Write every file the sorter loads, with the reference exporter's dtypes and orders
    (run_online_spikes.py:641-672, crop_methods.py:171-175)."""
    d = Path(out_dir)
    d.mkdir(parents=True, exist_ok=True)
    np.save(d / "templates.npy", np.ascontiguousarray(oss.templates, np.float32))
    np.save(d / "whiteningMat.npy", np.ascontiguousarray(oss.whitening, np.float32))
    np.save(d / "channelMap.npy", np.ascontiguousarray(oss.channel_map, np.int32))
    np.save(d / "templateMap.npy", np.ascontiguousarray(oss.template_map, np.int32))
    np.save(d / "Wall3.npy", np.ascontiguousarray(oss.Wall3, np.float32))
    np.save(d / "ctc.npy", np.ascontiguousarray(oss.ctc, np.float32))
    np.save(d / "wPCA.npy", np.ascontiguousarray(oss.wPCA, np.float32))
    np.save(d / "wPCA_permuted.npy", np.ascontiguousarray(oss.wPCA.T, np.float32))
    np.save(d / "preclustered_template_waveforms.npy", np.ascontiguousarray(oss.pre_wf, np.float32))
    # the exporter saves get_drift_matrix(...).T: a Fortran-ordered file whose raw bytes are M
    np.save(d / "drift_matrix.npy", np.ascontiguousarray(oss.drift, np.float32).T)
    np.save(d / "iCC.npy", np.ascontiguousarray(oss.iCC, np.int64))
    np.save(d / "iU.npy", np.ascontiguousarray(oss.iU, np.int64))
    np.save(d / "Ucc.npy", np.ascontiguousarray(oss.Ucc, np.float32))
    np.save(d / "hp_filter.npy", np.ascontiguousarray(oss.hp_filter, np.float32))
    np.save(d / "xc.npy", np.ascontiguousarray(oss.xc, np.float32))
    np.save(d / "yc.npy", np.ascontiguousarray(oss.yc, np.float32))
    np.save(d / "cluster_centroids.npy", np.ascontiguousarray(oss.centroids, np.float32))
    np.save(d / "cluster_centroids_pca.npy", np.ascontiguousarray(oss.centroids_pca, np.float32))
    np.save(d / "spike_templates.npy", np.ascontiguousarray(oss.spike_templates, np.int64))
    np.save(d / "spike_detection_templates.npy", np.ascontiguousarray(oss.spike_templates, np.int64))
    with open(d / "misc.txt", "w") as f:
        for k in ("nt0min", "numNearestChans", "Th_learned", "duplicate_spike_bins"):
            f.write(f"{k}:{oss.misc[k]}\n")
    return d


def cached_dataset(cfg: SynthConfig, root=None):
    """Build (or reuse) the recording + oss_input dir for ``cfg`` under a cache folder.

    Returns ``(oss_dir, data_int16[N, C], recording)``; the recording is rebuilt from the
    seed when the cache is missing.
    """
    root = Path(root or os.environ.get("LSS_SYNTH_CACHE", Path(__file__).resolve().parent.parent / "_synth_cache"))
    digest = hashlib.sha1(cfg.to_json().encode()).hexdigest()[:10]
    key = f"c{cfg.n_chan}_u{cfg.n_units}_n{cfg.n_samples}_s{cfg.seed}_{digest}"
    d = root / key
    rec = make_recording(cfg)
    if not (d / "oss_input" / "misc.txt").exists():
        oss = build_oss_input(rec)
        write_oss_input(oss, d / "oss_input")
    return d / "oss_input", rec.data, rec


def threshold_recording(n_rows: int, n_chan: int = 384, seed: int = 0, rate_hz: float = 40.0,
                        fs: float = 30000.0, chunk: int = 65536) -> np.ndarray:
    """Seeded raw int16 rows [n_rows][n_chan] for the threshold-crossing detector: a per-channel
    DC offset (SD 20) and Gaussian noise (SD 5-12 counts, unfiltered like the reference's input),
    plus negative biphasic spikes (peak lognormal around 90 counts) on five neighbouring channels,
    rate_hz per group of 8 channels.  Generated chunk by chunk to bound host memory."""
    rng = np.random.default_rng(seed)
    dc = rng.normal(0, 20, n_chan)
    sd = rng.uniform(5, 12, n_chan)
    out = np.empty((n_rows, n_chan), np.int16)
    L = 30
    wave = (-np.exp(-0.5 * ((np.arange(L) - 10) / 2.5) ** 2)
            + 0.35 * np.exp(-0.5 * ((np.arange(L) - 18) / 4.0) ** 2))
    spread = np.exp(-0.5 * np.arange(-2, 3) ** 2)
    for a in range(0, n_rows, chunk):
        b = min(n_rows, a + chunk)
        x = rng.standard_normal((b - a + L, n_chan), dtype=np.float32) * sd[None, :] + dc[None, :]
        n_sp = rng.poisson(rate_hz * n_chan / 8 * (b - a) / fs)
        t0 = rng.integers(0, b - a, n_sp)
        c0 = rng.integers(0, n_chan, n_sp)
        amp = rng.lognormal(np.log(90.0), 0.4, n_sp)
        for t, c, am in zip(t0, c0, amp):
            lo, hi = max(0, c - 2), min(n_chan, c + 3)
            x[t:t + L, lo:hi] += (am * wave)[:, None] * spread[lo - c + 2:hi - c + 2][None, :]
        out[a:b] = np.clip(np.rint(x[:b - a]), -32768, 32767).astype(np.int16)
    return out
