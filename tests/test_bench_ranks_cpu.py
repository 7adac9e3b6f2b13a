"""bench.py's multi-rank path without a GPU: two gloo ranks on 127.0.0.1 agree on the job time
(the slowest rank's) and on the whole-job rate (every rank's units over that time), as the driver's
torchrun launch needs; the reference arm's other ranks exit 0 without work."""
import os
import socket
import sys
import types
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(times[rank], world)
        q.put((rank, t, bench.whole_job_rate(1000.0, t, world)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    times = [0.25, 0.75]
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [0.75, 0.75]
    assert all(abs(g[2] - 2 * 1000.0 / 0.75) < 1e-9 for g in got)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(1.5, 1) == 1.5
    assert bench.whole_job_rate(300.0, 2.0, 1) == 150.0


def test_reference_arm_other_ranks_do_no_work(monkeypatch, capsys):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr(bench, "dataset", lambda *_: (_ for _ in ()).throw(AssertionError("rank 1 did work")))
    assert bench.run_reference(types.SimpleNamespace(seconds=1.0, steps=1, warmup=1, gpus=2)) == 0
    assert capsys.readouterr().out == ""
