"""The C-ABI library without a GPU: it builds, loads, exports every function the header
declares, its structs match the header layout, and the host-side loader rejects bad
oss_input directories with a status code (the reference calls exit(), SorterHelpers.cpp:36-39,
OnlineSpikesV2.cu:467-471)."""
import ctypes as ct
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from livespikesorter_gb300 import sorter, synth

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    return sorter.load_library()


@pytest.fixture(scope="module")
def small_oss(tmp_path_factory):
    cfg = synth.SynthConfig(n_chan=32, n_units=8, n_samples=4000, whiten_batch=1500, whiten_batches=2, seed=3)
    rec = synth.make_recording(cfg)
    d = tmp_path_factory.mktemp("oss") / "oss_input"
    synth.write_oss_input(synth.build_oss_input(rec), d)
    return d


def test_exports_every_declared_function(lib):
    names = sorter.header_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(sorter._SIGS)


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "lss_gb300.h"\n'
                   'int main(){printf("%zu %zu %zu %zu %zu\\n", sizeof(lss_params), sizeof(lss_spike),'
                   ' sizeof(lss_info), offsetof(lss_spike, pcfeat), offsetof(lss_params, mem_budget));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [ct.sizeof(sorter.Params), ct.sizeof(sorter.Spike), ct.sizeof(sorter.Info),
                   sorter.Spike.pcfeat.offset, sorter.Params.mem_budget.offset]


def test_other_headers_struct_layouts(tmp_path):
    """The proposal, payload and threshold-crossing structs as C sees them, against the ctypes
    mirrors (every field's offset and the size)."""
    from livespikesorter_gb300 import payload, proposal, threshold
    mirrors = [("lss_prop_train_params", "lss_proposal.h", proposal.TrainParams),
               ("lss_payload_header", "lss_payload.h", payload.PayloadHeader),
               ("lss_tc_params", "lss_threshold.h", threshold.TcParams),
               ("lss_tc_event", "lss_threshold.h", threshold.TcEvent)]
    lines = []
    for cname, _, py in mirrors:
        fields = [f for f, _ in py._fields_]
        lines.append('printf("%zu' + " %zu" * len(fields) + '\\n", sizeof(' + cname + ")"
                     + "".join(f", offsetof({cname}, {f})" for f in fields) + ");")
    incs = "".join(f'#include "{h}"\n' for h in sorted({h for _, h, _ in mirrors}))
    src = tmp_path / "layout.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n" + incs + "int main(){" + "".join(lines) + "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()
    for (cname, _, py), line in zip(mirrors, out):
        want = [ct.sizeof(py)] + [getattr(py, f).offset for f, _ in py._fields_]
        assert [int(v) for v in line.split()] == want, cname


def test_default_params(lib):
    p = sorter.default_params()
    assert p.abi_version == sorter.ABI_VERSION
    assert (p.batch_samples, p.max_iters, p.group_batches, p.dedup) == (1500, 50, 1, 1)


def _open_status(lib, d, **kw):
    p = sorter.default_params(**kw)
    h = ct.c_void_p()
    st = lib.lss_open(str(d).encode(), ct.byref(p), ct.byref(h))
    msg = (lib.lss_last_error(None) or b"").decode()
    if st == 0:
        lib.lss_close(h)
    return st, msg


def test_missing_dir_is_io_error(lib, tmp_path):
    st, msg = _open_status(lib, tmp_path / "nope")
    assert st == 2 and "misc.txt" in msg


def test_open_error_message_is_per_thread(lib, tmp_path):
    """lss_last_error(NULL) is the message of this thread's last failed call without a handle: a
    failure on another thread does not replace it."""
    import threading
    st, msg = _open_status(lib, tmp_path / "nope")
    assert st == 2 and "misc.txt" in msg
    other = {}

    def run():
        other["st"], other["msg"] = _open_status(lib, small := tmp_path / "also_missing_dir_x")
        other["dir"] = str(small)

    t = threading.Thread(target=run)
    t.start()
    t.join()
    assert other["st"] == 2 and "also_missing_dir_x" in other["msg"]
    again = (lib.lss_last_error(None) or b"").decode()
    assert again == msg


def test_missing_misc_key(lib, small_oss, tmp_path):
    d = tmp_path / "o"
    shutil.copytree(small_oss, d)
    (d / "misc.txt").write_text("nt0min:20\nnumNearestChans:10\n")
    st, msg = _open_status(lib, d)
    assert st == 3 and "Th_learned" in msg


def test_wrong_shape_is_format_error(lib, small_oss, tmp_path):
    d = tmp_path / "o"
    shutil.copytree(small_oss, d)
    w = np.load(d / "Wall3.npy")
    np.save(d / "Wall3.npy", w[:, :, :-1])
    st, msg = _open_status(lib, d)
    assert st == 3 and "Wall3" in msg


def test_truncated_npy_is_format_error(lib, small_oss, tmp_path):
    d = tmp_path / "o"
    shutil.copytree(small_oss, d)
    raw = (d / "ctc.npy").read_bytes()
    (d / "ctc.npy").write_bytes(raw[: len(raw) // 2])
    st, msg = _open_status(lib, d)
    assert st == 3 and "ctc" in msg


def test_validator_without_a_gpu(lib, small_oss, tmp_path):
    """lss_validate_oss_input: the dimensions of a good directory; for broken ones the status and
    message lss_open gives; the command-line tool's exit status."""
    from livespikesorter_gb300 import validate
    info = sorter.validate_oss_input(small_oss)
    w = np.load(small_oss / "Wall3.npy")
    assert (info.C, info.T, info.K) == (w.shape[2], w.shape[0], w.shape[1])
    assert info.nt == np.load(small_oss / "wPCA.npy").shape[1] and info.th == pytest.approx(8.0)
    assert info.device_bytes == 0 and info.NT == 0
    assert validate.main([str(small_oss)]) == 0
    broken = []
    d = tmp_path / "shape"
    shutil.copytree(small_oss, d)
    np.save(d / "Wall3.npy", w[:, :, :-1])
    broken.append(d)
    d = tmp_path / "misc"
    shutil.copytree(small_oss, d)
    (d / "misc.txt").write_text("nt0min:20\nnumNearestChans:10\n")
    broken.append(d)
    d = tmp_path / "truncated"
    shutil.copytree(small_oss, d)
    raw = (d / "ctc.npy").read_bytes()
    (d / "ctc.npy").write_bytes(raw[: len(raw) // 2])
    broken.append(d)
    broken.append(tmp_path / "missing")
    for d in broken:
        with pytest.raises(sorter.SorterError) as e:
            sorter.validate_oss_input(d)
        st, msg = _open_status(lib, d)
        assert e.value.status == st and msg in str(e.value)
    assert validate.main([str(small_oss), str(broken[0])]) == 1


def test_bad_params_rejected(lib, small_oss):
    st, _ = _open_status(lib, small_oss, batch_samples=0)
    assert st == 1
    p = sorter.default_params()
    p.abi_version = 99
    h = ct.c_void_p()
    assert lib.lss_open(str(small_oss).encode(), ct.byref(p), ct.byref(h)) == 1


def test_null_handles_are_rejected(lib):
    n = ct.c_int64()
    assert lib.lss_push_batch(None, None, 0, -1) == 1
    assert lib.lss_poll(None, None, 0, ct.byref(n)) == 1
    assert lib.lss_close(None) == 1


def test_no_gpu_open_fails_cleanly(lib, small_oss):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    st, msg = _open_status(lib, small_oss)
    assert st == 4, msg   # LSS_ERR_CUDA, no crash and no CPU fallback
