"""lss_match_noalloc: the matching loop on caller-owned device buffers, for callers that cannot
allocate device memory when they sort (a real-time acquisition thread that must not wait on the
allocator, code confined to another framework's memory pool).  Its spikes and residual must
equal the library's own window path (lss_sort_windows / lss_debug_stage) on two calls in a row:
the second call runs on the scratch array the first one left behind.

Collected last on purpose (file name), so a run that stops at the first failure has already run
every other test; it also passes on its own in a fresh process."""
import ctypes as ct

import numpy as np
import pytest

from livespikesorter_gb300 import sorter

from lss_testutil import agreement, write_oss_from_arrays

pytestmark = pytest.mark.gpu

CAP = 4096


def _run_noalloc(lib, torch, B0, X0, ctcP, pre_wf, nm, th, W, T, C, nt, max_iters):
    dev = torch.device("cuda:0")
    B = torch.from_numpy(B0.copy()).to(dev)
    X = torch.from_numpy(X0.copy()).to(dev)
    tc = torch.from_numpy(ctcP).to(dev)
    wf = torch.from_numpy(pre_wf).to(dev)
    tn = torch.from_numpy(nm).to(dev)
    n = torch.zeros(1, dtype=torch.int32, device=dev)
    sw = torch.full((CAP,), -1, dtype=torch.int32, device=dev)
    stt = torch.full((CAP,), -1, dtype=torch.int32, device=dev)
    sa = torch.zeros(CAP, dtype=torch.float32, device=dev)
    si = torch.full((CAP,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.lss_match_noalloc(B.data_ptr(), X.data_ptr(), tc.data_ptr(), wf.data_ptr(), tn.data_ptr(), ct.c_float(th),
                               W, T, C, nt, max_iters, n.data_ptr(), sw.data_ptr(), stt.data_ptr(), sa.data_ptr(),
                               si.data_ptr(), CAP, ct.c_void_p(stream.cuda_stream))
    assert rc == 0, (lib.lss_last_error(None) or b"").decode()
    torch.cuda.synchronize(dev)
    k = int(n.item())
    assert k >= 0, f"the matching kernel reported a fault (status bits {-k})"
    assert 0 < k <= CAP
    return (sw[:k].cpu().numpy(), stt[:k].cpu().numpy(), sa[:k].cpu().numpy(), si[:k].cpu().numpy(),
            X.cpu().numpy())


def test_noalloc_matches_window_path_twice(golden_dir, tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    z = np.load(golden_dir / "ks_window.npz")
    d = write_oss_from_arrays(z, tmp_path / "oss_input")
    max_iters = int(z["max_iters"])
    window = z["window"]
    with sorter.OnlineSorter(d, max_iters=max_iters) as s:
        (ref,) = s.sort_windows(window)                              # the existing entry point
        X0 = s.debug_stage(window, sorter.STAGE_PREPROCESSED)
        B0 = s.debug_stage(window, sorter.STAGE_SCORES)
        Xres_ref = s.debug_stage(window, sorter.STAGE_RESIDUAL)
        info = s.get_info()
        th, T, C, nt, nt0 = info.th, info.T, info.C, info.nt, info.nt0min
    W = window.shape[0]
    ctcP = np.ascontiguousarray(z["ctc"].transpose(1, 2, 0))        # [s][l][t] = ctc[t][s][l]
    nm = (z["Wall3"].astype(np.float64) ** 2).sum((1, 2)).astype(np.float32)
    pre_wf = np.ascontiguousarray(z["pre_wf"], np.float32)
    lib = sorter.load_library()

    runs = [_run_noalloc(lib, torch, B0, X0, ctcP, pre_wf, nm, th, W, T, C, nt, max_iters) for _ in range(2)]
    for w, t, a, it, X in runs:
        time = w.astype(np.int64) - nt // 2 + nt0
        frac, amp_ok, amax = agreement(ref["time"], ref["tmpl"], ref["amp"], time, t, a)
        assert frac == 1.0 and amp_ok == 1.0, (frac, amp_ok, amax)
        assert len(w) == len(ref)
        # spikes come out in (iteration, sample) order
        assert np.all(np.diff(it) >= 0)
        scale = np.abs(Xres_ref).max()
        assert np.abs(X - Xres_ref).max() <= 5e-5 * scale
    for f in range(5):
        np.testing.assert_array_equal(runs[0][f], runs[1][f])


def test_noalloc_rejects_oversized_window():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = sorter.load_library()
    buf = torch.zeros(64, device="cuda:0")
    p = buf.data_ptr()
    too_big = 16384 + 1
    rc = lib.lss_match_noalloc(p, p, p, p, p, ct.c_float(8.0), too_big, 4, 4, 61, 10, p, p, p, p, p, 1, None)
    assert rc == 1
    assert b"16384" in lib.lss_last_error(None)
