"""ORACLE (timing form) -- test infrastructure, not product code.  Only tests/ and bench.py's
CPU-baseline / reference legs may import this module.

The same restatement of the reference's Kilosort 4.0.13 per-batch CPU path as ``ks_oracle`` (whose
docstrings cite the vendored lines), written with torch CPU tensor operations in float32 the way
the vendored code runs -- ``BinaryFiltered.filter`` (KS/io.py:757-790), ``run_matching``
(KS/template_matching.py:128-202) with the PC features (:50-51) and positions
(KS/postprocessing.py:33-46) -- so that the CPU baseline runs at the speed of the reference's own
torch path on the host's cores (the vendored modules cannot be shipped with this repository).
``tests/test_ks_torch_cpu.py`` checks it against ``ks_oracle`` on the same inputs.
"""
from __future__ import annotations

import numpy as np


def _t():
    import torch
    return torch


def preprocess(window_CW, oss, hp_kernel_fft=None):
    """[C, W] int16 / float window -> [C, W] float32: mean removal, lower-median CAR, the circular
    zero-phase high-pass (FFT of the cropped filter, fftshift), then (M @ Wrot)."""
    torch = _t()
    from . import ks_oracle as ko
    X = torch.as_tensor(np.asarray(window_CW, np.float32))
    X = X - X.mean(1, keepdim=True)
    X = X - torch.median(X, 0)[0]     # torch.median: the lower median, as the vendored filter
    W = X.shape[1]
    if hp_kernel_fft is None:
        h = torch.as_tensor(ko.fft_highpass_kernel(oss.hp_filter.astype(np.float64), W).astype(np.float32))
        hp_kernel_fft = torch.fft.fft(h)
    X = torch.real(torch.fft.ifft(torch.fft.fft(X) * torch.conj(hp_kernel_fft)))
    X = torch.fft.fftshift(X, dim=-1)
    WD = torch.as_tensor((oss.drift.astype(np.float64) @ oss.whitening.astype(np.float64)).astype(np.float32))
    return WD @ X


class Matcher:
    """Fixed operands of one oss_input (float32 torch tensors), reused across batches."""

    def __init__(self, oss):
        torch = _t()
        self.oss = oss
        self.U = torch.as_tensor(np.asarray(oss.Wall3, np.float32))          # [T, K, C]
        self.W = torch.as_tensor(np.asarray(oss.wPCA, np.float32))           # [K, nt]
        self.ctc = torch.as_tensor(np.asarray(oss.ctc, np.float32))          # [T, T, 2nt+1]
        self.nm = (self.U ** 2).sum((1, 2))
        self.Th = float(oss.th_learned)
        nt = self.W.shape[1]
        self.trange = torch.arange(-nt, nt + 1)
        self.tiwave = torch.arange(-(nt // 2), nt // 2 + 1)
        self.iCC = torch.as_tensor(np.asarray(oss.iCC, np.int64))
        self.iU = torch.as_tensor(np.asarray(oss.iU, np.int64))
        self.Ucc = torch.as_tensor(np.asarray(oss.Ucc, np.float32))
        self.xc = torch.as_tensor(np.asarray(oss.xc, np.float32))
        self.yc = torch.as_tensor(np.asarray(oss.yc, np.float32))

    def run(self, X, max_iters: int = 50):
        """-> (st [S, 2] (sample, template), amps [S], Xres [C, W], tF [S, nC, K], xs, ys)."""
        torch = _t()
        U, Wb, ctc, nm = self.U, self.W, self.ctc, self.nm
        T, K, C = U.shape
        nt = Wb.shape[1]
        Xres = X.clone()
        Bpc = torch.nn.functional.conv1d(X.unsqueeze(1), Wb.unsqueeze(1), padding=nt // 2)   # [C, K, W]
        B = torch.einsum("tkc,ckw->tw", U, Bpc)
        st_l, amp_l = [], []
        Th2 = self.Th ** 2
        for _ in range(max_iters):
            Cf = torch.relu(B) ** 2 / nm.unsqueeze(-1)
            Cf[:, :nt] = 0
            Cf[:, -nt:] = 0
            Cfmax, imax = torch.max(Cf, 0)
            Cmax = torch.nn.functional.max_pool1d(Cfmax.unsqueeze(0).unsqueeze(0), 2 * nt + 1, stride=1,
                                                  padding=nt)[0, 0]
            xs = torch.nonzero((Cmax > Th2) & (torch.abs(Cmax - Cfmax) < 1e-9))[:, 0]
            if len(xs) == 0:
                break
            iY = imax[xs]
            amp = B[iY, xs] / nm[iY]
            st_l.append(torch.stack([xs, iY], 1))
            amp_l.append(amp)
            for j in range(2):
                ix, iy, a = xs[j::2], iY[j::2], amp[j::2]
                if len(ix) == 0:
                    continue
                wf = torch.einsum("nkc,kl->cnl", U[iy], Wb)                      # [C, n, nt]
                Xres[:, ix[:, None] + self.tiwave[None, :]] -= a[None, :, None] * wf
                B[:, ix[:, None] + self.trange[None, :]] -= a[None, :, None] * ctc[:, iy, :]
        if not st_l:
            e = torch.zeros(0)
            return torch.zeros((0, 2), dtype=torch.int64), e, Xres, torch.zeros((0, self.iCC.shape[0], K)), e, e
        st = torch.cat(st_l)
        amps = torch.cat(amp_l)
        chans = self.iCC[:, self.iU[st[:, 1]]]                                   # [nC, S]
        times = st[:, 0][:, None] + self.tiwave[None, :]
        seg = Xres[chans[:, :, None], times[None, :, :]]                         # [nC, S, nt]
        tF = (seg @ Wb.T + amps[None, :, None] * self.Ucc[:, st[:, 1]]).permute(1, 0, 2)
        tmass = (tF ** 2).sum(-1)
        tmass = tmass / tmass.sum(1, keepdim=True)
        chs = chans.T
        xs = (self.xc[chs] * tmass).sum(1)
        ys = (self.yc[chs] * tmass).sum(1)
        return st, amps, Xres, tF, xs, ys
