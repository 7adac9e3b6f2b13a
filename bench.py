#!/usr/bin/env python
"""Throughput and latency of the per-batch sorting path on GB300.

Workload (the streamed drop-in case): 384 channels at 30 kHz, 500 templates (6 PCs, nt = 61),
a seeded 60 s recording with a 0-20 um rigid drift cut into 1500-sample batches with nt of
context on each side, 50 matching iterations, FP32 arithmetic.  One step = one group of
``--group`` consecutive batches through preprocessing, projection, the matching loop and
PC features.

* ``value``   device throughput (ch*samples/s of new samples) with the recording resident in
              HBM, timed with CUDA events on the sorter's stream, max over ranks;
* ``e2e``     the same through the public C ABI from host int16 buffers (lss_push_batch /
              lss_poll), host-to-device copies and spike read-back inside the timed region;
* ``latency`` per-batch push-to-spikes wall time with one batch per launch (p50 / p99);
* ``roofline`` of the dominant kernel from per-stage CUDA events;
* ``cpu_baseline`` the float32 CPU oracle port of the same batches on the host cores.

``--impl reference`` times the CPU oracle port (the reference's Kilosort CPU path restated)
on the same workload.

``--serving`` measures several probe streams on one GPU at once (one handle and one host thread
per stream, each handle on its own CUDA stream): eight streams of uneven size (96/192/384
channels, 64-1000 templates, 750-3000-sample batches) paced at 30 kHz with +/-20 % jitter
(per-batch push-to-spikes latency p50/p99), the same streams unpaced (aggregate ch*samples/s),
and eight 384-channel / 500-template streams unpaced (aggregate, as a multiple of real time).

``--path proposal`` trains the learned proposal gate on the device (labels from the plain matcher on
the first ``--prop-train-windows`` windows of the recording), then reports, on held-out seeds of
the same units at 5-40 Hz, the fraction of the plain matcher's spikes the gated sorter keeps, the
fraction of (neighbourhood, window) cells it leaves open, and device throughput gated and plain.

``--path tc`` measures the reference's other sorter, threshold crossing, instead: 384 channels of
raw int16 at 30 kHz, one step = one push of ``--tc-rows`` rows (20 s, 461 MB, larger than L2)
tested against 3 x the per-channel median; same JSON keys, roofline of the count kernel (2 bytes
read per channel-sample).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NT = 1500
METRIC = "ch*samples/s & p99 batch latency, chosen vs plain FP32 at >=99.5% spike match"
UNIT = "ch*samples/s"
SPIKE_REC_BYTES = 288


def args_():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=18)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--seconds", type=float, default=60.0)
    ap.add_argument("--group", type=int, default=64, help="batches per step")
    ap.add_argument("--latency-batches", type=int, default=200)
    ap.add_argument("--cpu-sample", type=int, default=6, help="batches timed on the CPU oracle")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--match-variant", type=int, default=0, help="0 auto, 1 scores in L2, 2 scores in SMEM")
    ap.add_argument("--match-keep", type=int, default=0,
                    help="match_keep of the measured path (0 = Kilosort's loop over every template)")
    ap.add_argument("--match-keep-wide", type=int, default=0,
                    help="match_keep_wide of the measured path (crowded samples' list length; 0 = fixed lists)")
    ap.add_argument("--match-keep-crowd", type=float, default=0.5,
                    help="match_keep_crowd of the measured path (crowded: the match_keep-th largest Cf above this x Th^2)")
    ap.add_argument("--gemm-path", type=int, default=0,
                    help="0 tcgen05 FP32 (3xTF32), 1 FP32 SIMT, 2 tcgen05 with TF32 data (two products)")
    ap.add_argument("--no-tier", action="store_true", help="skip the chosen-tier measurement")
    ap.add_argument("--chosen-only", default=None, help="measure only this chosen-path candidate beside fp32")
    ap.add_argument("--chosen-seconds", type=float, default=4.0,
                    help="signal per stream of the 8-stream chosen-path measurement (0 = skip it)")
    ap.add_argument("--path", default="sort", choices=["sort", "tc", "proposal"],
                    help="sort = template matching (default); tc = threshold crossing; proposal = the learned "
                         "proposal gate (train, then recall / cells closed / throughput against the plain matcher)")
    ap.add_argument("--prop-train-windows", type=int, default=256, help="batch windows the gate trains on")
    ap.add_argument("--prop-steps", type=int, default=400, help="Adam steps of 64 examples")
    ap.add_argument("--tc-rows", type=int, default=600_000, help="rows per threshold-crossing push")
    ap.add_argument("--serving", action="store_true", help="several concurrent probe streams")
    ap.add_argument("--serving-seconds", type=float, default=8.0, help="signal per stream")
    return ap.parse_args()


def dataset(seconds: float):
    from livespikesorter_gb300 import synth
    cfg = synth.config_stream(seconds=seconds, seed=1)
    oss_dir, data, _ = synth.cached_dataset(cfg)
    return cfg, oss_dir, data


def workload_config(a, cfg, group):
    return {"workload": "drop-in streaming, 384 ch x 30 kHz int16, 500 templates, 1500-sample batches "
                        "+ 2*61 context, 50 iterations, FP32",
            "channels": cfg.n_chan, "templates": cfg.n_units, "batch_samples": NT, "nt": cfg.nt,
            "recording_s": a.seconds, "batches_per_step": group, "max_iters": 50,
            "l2": "inputs larger than L2: every step reads a fresh slice of the HBM-resident recording "
                  "and streams > 1 GB of intermediates",
            "parallelism": "replicas" if a.gpus > 1 else "single"}


# -------------------------------------------------------------------------------------------
# CPU oracle port (reference arm and cpu_baseline)
# -------------------------------------------------------------------------------------------
def cpu_oracle_rate(data, oss_dir, n_batches, warm=1):
    """The reference's Kilosort CPU path as the torch (float32) form of the oracle runs it -- the
    vendored filter + run_matching restated with torch CPU operations, plus PC features and
    positions -- on the host's cores (torch.set_num_threads(os.cpu_count())), one batch at a time;
    returns (new ch*samples per second, per-batch seconds)."""
    import torch
    from oracle import ks_oracle as ko
    from oracle import ks_torch
    torch.set_num_threads(os.cpu_count())
    oss = ko.load_oss_input(oss_dir)
    nt = oss.wPCA.shape[1]
    nbat = ko.n_batches(data.shape[0], NT)
    ids = [1 + (i * 7) % (nbat - 2) for i in range(n_batches + warm)]
    matcher = ks_torch.Matcher(oss)
    times = []
    for i, ib in enumerate(ids):
        X = ko.padded_batch(data, ib, NT, nt)
        t0 = time.perf_counter()
        matcher.run(ks_torch.preprocess(X, oss), max_iters=50)
        dt = time.perf_counter() - t0
        if i >= warm:
            times.append(dt)
    total = sum(times)
    return n_batches * NT * data.shape[1] / total, times


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cfg, oss_dir, data = dataset(a.seconds)
    t0 = time.perf_counter()
    rate, times = cpu_oracle_rate(data, oss_dir, a.steps, warm=a.warmup)
    cores = os.cpu_count()
    line = {"metric": METRIC, "value": rate, "unit": UNIT, "impl": "reference", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * float(np.mean(times)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator, shapes of the named config)",
            "config": workload_config(a, cfg, 1),
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{a.steps} batches of 1500 new samples (+2*61 context) of the 60 s "
                                       f"recording through the torch float32 form of the oracle (Kilosort "
                                       f"filter + run_matching + xfeat + positions, the vendored path's torch "
                                       f"operations), {cores} host threads"},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t0}
    print(json.dumps(line))
    return 0


# -------------------------------------------------------------------------------------------
# GPU arm
# -------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once nvidia-smi has initialised and sampled once: its start-up
            # competes with the timed launches otherwise
            t_end = time.perf_counter() + 3.0
            while not self.lines and self.proc.poll() is None and time.perf_counter() < t_end:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        load = sorted(sm)[len(sm) // 4:] or sm
        return {"sm_mhz": float(np.median(load)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops_sustained", 1700.0), "measured"
    return 6800.0, 1700.0, "fallback"


def roofline(stage_ms, n_groups, group, C, T, K, nt, W, ntaps, spikes_per_batch, mean_reach=None):
    """Achieved vs peak for the dominant kernel (per-launch algorithmic work / mean duration).  For
    the matching loop the algorithmic bytes are one score scan plus, per spike, the ctc read and score
    read-modify-write of the templates it updates (mean_reach of them on average -- all T in Kilosort's
    dense subtraction); the residual is not part of the sorting path (the features come from the
    convolution)."""
    hbm, tflops, src = peaks()
    per = {k: v / max(n_groups, 1) for k, v in stage_ms.items()}
    kern = max((k for k in per if k not in ("h2d", "d2h")), key=lambda k: per[k])
    ms = per[kern]
    if kern == "project":
        work, unit, bound, peak = 2.0 * T * K * C * W * group / 1e12, "TFLOP/s", "tensor", tflops
    elif kern == "highpass":
        work, unit, bound, peak = 2.0 * C * W * ntaps * group / 1e12, "TFLOP/s", "tensor", tflops
    elif kern == "whiten":
        work, unit, bound, peak = 2.0 * C * C * W * group / 1e12, "TFLOP/s", "tensor", tflops
    elif kern == "basis_conv":
        work, unit, bound, peak = 2.0 * C * K * nt * W * group / 1e12, "TFLOP/s", "tensor", tflops
    elif kern == "match":
        reach = T if mean_reach is None else mean_reach
        per_spike = reach * (2 * nt + 1) * (4 + 8)
        work = group * (4.0 * T * W + spikes_per_batch * per_spike) / 1e9
        dense = group * (4.0 * T * W + spikes_per_batch * T * (2 * nt + 1) * 12) / 1e9
        unit, bound, peak = "GB/s", "hbm", hbm
    else:
        work = group * (2.0 * W * C + 4.0 * W * C) / 1e9
        unit, bound, peak = "GB/s", "hbm", hbm
    achieved = work / (ms / 1e3)
    # DRAM bytes (read + write) per batch of each stage's kernel on the FP32 path from ncu captures of the
    # 64-batch group (profiles/match_kernel_interleaved_64batches.md,
    # profiles/preprocess_and_gemm_kernels_64batches.md), scaled to this launch's batches
    traffic_per_batch = {"match": 8.477e9 / 64, "project": 2.216e9 / 64, "basis_conv": 2.172e9 / 64,
                         "highpass": 0.796e9 / 64, "whiten": 0.597e9 / 64, "car": 0.515e9 / 64}
    traffic = traffic_per_batch.get(kern)
    out = {"kernel": kern, "bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
           "frac": achieved / peak, "peak_source": src, "algorithmic_gb_per_launch": work if unit == "GB/s" else None,
           "traffic": None if traffic is None else traffic * group,
           "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, 64-batch capture, scaled by batches",
           "ms_per_launch": ms, "stage_ms_per_launch": per}
    if traffic is not None and unit == "GB/s":
        # the DRAM side of the same launch: measured traffic over the live duration
        out["dram_gbs"] = traffic * group / 1e9 / (ms / 1e3)
        out["dram_frac"] = out["dram_gbs"] / peak
        if achieved > out["dram_gbs"]:
            out["note"] = ("algorithmic bytes exceed the DRAM traffic: ctc and score rows are re-read from L2, "
                           "so frac can pass 1; dram_frac is the HBM side")
    if kern == "match":
        out["mean_templates_updated_per_spike"] = reach
        out["dense_kilosort_gb_per_launch"] = dense
        out["dense_kilosort_gbs"] = dense / (ms / 1e3)
    return out


def spike_agreement(ref, got, tol=1):
    """Fraction of ref spikes with a got spike of the same template within tol samples, and the
    fraction of those whose amplitudes agree within 1e-3 relative (each got spike used once)."""
    if len(ref) == 0:
        return 1.0, 1.0
    order = np.lexsort((got["time"], got["tmpl"]))
    gt, gk, ga = got["time"][order], got["tmpl"][order], got["amp"][order]
    used = np.zeros(len(gt), bool)
    matched = amp_ok = 0
    for t, k, amp in zip(ref["time"], ref["tmpl"], ref["amp"]):
        lo = np.searchsorted(gk, k, "left")
        hi = np.searchsorted(gk, k, "right")
        i0 = lo + np.searchsorted(gt[lo:hi], t - tol, "left")
        i1 = lo + np.searchsorted(gt[lo:hi], t + tol, "right")
        for i in range(i0, i1):
            if not used[i]:
                used[i] = True
                matched += 1
                amp_ok += abs(ga[i] - amp) <= 1e-3 * max(abs(amp), 1e-12)
                break
    return matched / len(ref), amp_ok / max(1, matched)


def max_over_ranks(x: float, world: int, device=None) -> float:
    """The largest of every rank's x: a replicated job takes its slowest replica's time (all
    ranks of the process group call this; with world 1 it is x)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, seconds: float, world: int) -> float:
    """Units of every replica over the job's (slowest replica's) time."""
    return world * units_per_rank / seconds


def run_gpu(a):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
        torch.cuda.set_device(local)
    dev = local
    torch.cuda.set_device(dev)
    from livespikesorter_gb300 import sorter

    cfg, oss_dir, data = dataset(a.seconds)
    C, nt, T, K = cfg.n_chan, cfg.nt, cfg.n_units, cfg.n_pcs
    W = NT + 2 * nt
    G = a.group
    n_usable = (data.shape[0] - 2 * nt) // NT
    n_groups = max(1, n_usable // G)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- device-resident throughput -------------------------------------------------------
    d_data = torch.from_numpy(data).to(f"cuda:{dev}")
    base_ptr = d_data.data_ptr()
    row_bytes = C * 2
    s = sorter.OnlineSorter(oss_dir, device=dev, batch_samples=NT, max_iters=50, group_batches=G, profile=1,
                           match_variant=a.match_variant, gemm_path=a.gemm_path, match_keep=a.match_keep,
                           match_keep_wide=a.match_keep_wide if a.match_keep else 0,
                           match_keep_crowd=a.match_keep_crowd)
    ext = torch.cuda.ExternalStream(s.cuda_stream(), device=f"cuda:{dev}")
    spikes_seen = [0]

    def step(i):
        # cycle over the recording; stream times keep increasing (a continuous stream)
        g0 = (i % n_groups) * G
        s.push_device_span(base_ptr + g0 * NT * row_bytes, G, i * G * NT)

    def drain(srt):
        n = srt.pending()
        srt.poll(max(n, 1))
        return n

    for i in range(a.warmup):
        step(i)
    drain(s)
    t_base, n_base = s.stage_times()
    launches_per_step = s.kernel_launches()
    barrier()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        with torch.cuda.stream(ext):
            e0.record(ext)
        for i in range(a.steps):
            step(a.warmup + i)
        with torch.cuda.stream(ext):
            e1.record(ext)
        e1.synchronize()
    ms = e0.elapsed_time(e1)
    timed_spikes = s.poll(max(s.pending(), 1))
    spikes_seen[0] = len(timed_spikes)
    torch.cuda.synchronize(dev)
    ms = max_over_ranks(ms, world, f"cuda:{dev}")
    units = a.steps * G * NT * C
    value = whole_job_rate(units, ms / 1e3, world)
    t_all, n_all = s.stage_times()
    stage = {k: t_all[k] - t_base[k] for k in t_all}
    n_timed = n_all - n_base
    spikes_per_batch = spikes_seen[0] / max(1, a.steps * G)
    ntaps = 885   # the FIR the library cuts from this filter: taps beyond are < 1e-8 of the centre tap
    roof = roofline(stage, n_timed, G, C, T, K, nt, W, ntaps, spikes_per_batch)
    s.close()

    obuf = np.zeros(1 << 16, sorter.SPIKE_DTYPE)

    def batch_latency(path, n, keep=0):
        """push-to-spikes wall time of single 1500-sample batches (one batch per launch)"""
        s3 = sorter.OnlineSorter(oss_dir, device=dev, batch_samples=NT, max_iters=50, group_batches=1, profile=1,
                                 match_variant=a.match_variant, gemm_path=path, match_keep=keep,
                                 match_keep_wide=a.match_keep_wide if keep else 0,
                                 match_keep_crowd=a.match_keep_crowd)
        lat = []
        s3.push(data[:NT + 2 * nt], 0)
        drain(s3)
        p = NT + 2 * nt
        for i in range(n + 5):
            if p + NT > data.shape[0]:
                break
            t1 = time.perf_counter()
            s3.push(data[p: p + NT])
            s3.poll(out=obuf)
            if i >= 5:
                lat.append(1e3 * (time.perf_counter() - t1))
            p += NT
        st3, ng3 = s3.stage_times()
        s3.close()
        return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "batches": len(lat), "batch_ms_of_signal": 1e3 * NT / 30000.0,
                "path": "lss_push_batch of 1500 new samples -> lss_poll, group_batches=1",
                "stage_ms_per_batch": {k: v / max(ng3, 1) for k, v in st3.items()}}

    # ---- the chosen tier at group throughput: every candidate path on the same 64-batch groups ------
    # (device-resident input), its spike agreement with the FP32 path on the same 256 batches; the
    # tier is the fastest candidate at >= 99.5 % agreement with >= 99.5 % of amplitudes within 1e-3
    tier = None
    if a.gemm_path == 0 and not a.no_tier:
        n_rows = min(data.shape[0], 256 * NT + 2 * nt)
        with sorter.OnlineSorter(oss_dir, device=dev, batch_samples=NT, max_iters=50, group_batches=G,
                                 match_variant=a.match_variant) as sa:
            ref_spikes = sa.sort_stream(data[:n_rows])
        rows = []
        for label, opts, arith in CHOSEN_CANDIDATES[1:]:
            st = sorter.OnlineSorter(oss_dir, device=dev, batch_samples=NT, max_iters=50, group_batches=G, profile=1,
                                     match_variant=a.match_variant, **opts)
            ext2 = torch.cuda.ExternalStream(st.cuda_stream(), device=f"cuda:{dev}")

            def step2(i, st=st):
                g0 = (i % n_groups) * G
                st.push_device_span(base_ptr + g0 * NT * row_bytes, G, i * G * NT)

            for i in range(a.warmup):
                step2(i)
            drain(st)
            tb, nb0 = st.stage_times()
            torch.cuda.synchronize(dev)
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(ext2):
                f0.record(ext2)
            for i in range(a.steps):
                step2(a.warmup + i)
            with torch.cuda.stream(ext2):
                f1.record(ext2)
            f1.synchronize()
            ms2 = f0.elapsed_time(f1)
            drain(st)
            ta, na = st.stage_times()
            st.close()
            with sorter.OnlineSorter(oss_dir, device=dev, batch_samples=NT, max_iters=50, group_batches=G,
                                     match_variant=a.match_variant, **opts) as sa:
                got = sa.sort_stream(data[:n_rows])
            frac, amp_ok = spike_agreement(ref_spikes, got)
            rows.append({"label": label, **opts, "arithmetic": arith,
                         "value": a.steps * G * NT * C / (ms2 / 1e3), "unit": UNIT, "ms_per_step": ms2 / a.steps,
                         "speedup_vs_fp32": ms / ms2,
                         "stage_ms_per_launch": {k: (ta[k] - tb[k]) / max(1, na - nb0) for k in ta},
                         "agreement_vs_fp32": {"batches": (n_rows - 2 * nt) // NT, "spikes_fp32": int(len(ref_spikes)),
                                               "spikes_tier": int(len(got)), "matched": frac,
                                               "amp_within_1e-3": amp_ok}})
        ok = [r for r in rows if r["agreement_vs_fp32"]["matched"] >= 0.995 and
              r["agreement_vs_fp32"]["amp_within_1e-3"] >= 0.995]
        best = max(ok, key=lambda r: r["value"]) if ok else None
        if best is not None:
            tier = {**best, "rule": "fastest candidate at group throughput with >= 99.5 % spike agreement with the "
                                    "FP32 path and >= 99.5 % of amplitudes within 1e-3 (same template, |dt| <= 1)",
                    "latency": {k: v for k, v in batch_latency(best["gemm_path"], min(a.latency_batches, 100),
                                                               best["match_keep"]).items()
                                if k in ("p50_ms", "p99_ms", "batches")},
                    "candidates": [{k: r[k] for k in ("label", "value", "speedup_vs_fp32", "agreement_vs_fp32")}
                                   for r in rows]}
    # ---- the stateful high-pass mode beside the zero-phase one ----------------------------------
    stateful = None
    if a.gemm_path == 0 and not a.no_tier:
        ss = sorter.OnlineSorter(oss_dir, device=dev, batch_samples=NT, max_iters=50, group_batches=G, profile=1,
                                 match_variant=a.match_variant, highpass_mode=1)
        ext3 = torch.cuda.ExternalStream(ss.cuda_stream(), device=f"cuda:{dev}")
        for i in range(a.warmup):
            ss.push_device_span(base_ptr + (i % n_groups) * G * NT * row_bytes, G, i * G * NT)
        drain(ss)
        tb, nb0 = ss.stage_times()
        torch.cuda.synchronize(dev)
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(ext3):
            f0.record(ext3)
        for i in range(a.warmup, a.warmup + a.steps):
            # consecutive spans of the recording: the filter state carries from group to group
            ss.push_device_span(base_ptr + (i % n_groups) * G * NT * row_bytes, G, i * G * NT)
        with torch.cuda.stream(ext3):
            f1.record(ext3)
        f1.synchronize()
        ms3 = f0.elapsed_time(f1)
        drain(ss)
        ta, na = ss.stage_times()
        ss.close()
        n_rows = min(data.shape[0], 256 * NT + 2 * nt)
        got = {}
        for mode in (0, 1):
            with sorter.OnlineSorter(oss_dir, device=dev, batch_samples=NT, max_iters=50, group_batches=G,
                                     match_variant=a.match_variant, highpass_mode=mode) as sa:
                got[mode] = sa.sort_stream(data[:n_rows])
        frac, amp_ok = spike_agreement(got[0], got[1])
        per = {k: (ta[k] - tb[k]) / max(1, na - nb0) for k in ta}
        stateful = {"highpass_mode": 1, "value": a.steps * G * NT * C / (ms3 / 1e3), "unit": UNIT,
                    "ms_per_step": ms3 / a.steps,
                    "filter": "Butterworth 3rd order 300 Hz high-pass, second-order sections run forward, FP32 state "
                              "carried across groups; median CAR after it",
                    "stage_ms_per_launch": per,
                    "filter_and_car_ms_per_launch": per.get("colsum", 0) + per.get("car", 0) + per.get("highpass", 0),
                    "spikes_vs_zero_phase": {"batches": (n_rows - 2 * nt) // NT, "spikes_zero_phase": int(len(got[0])),
                                             "spikes_stateful": int(len(got[1])), "matched": frac,
                                             "amp_within_1e-3": amp_ok,
                                             "note": "different filters (causal vs zero-phase): agreement is not "
                                                     "expected to be 1; each mode is checked against its own float64 "
                                                     "oracle in the tests"}}
    del d_data

    # ---- end to end through the host API ---------------------------------------------------
    s2 = sorter.OnlineSorter(oss_dir, device=dev, batch_samples=NT, max_iters=50, group_batches=G,
                             match_variant=a.match_variant, gemm_path=a.gemm_path, match_keep=a.match_keep,
                             match_keep_wide=a.match_keep_wide if a.match_keep else 0,
                           match_keep_crowd=a.match_keep_crowd)
    chunk = G * NT
    pos = [0]
    # the caller's rows live in pinned host memory (the e2e contract); the API copies page-locked
    # rows straight into the pending group's device rows on its copy stream
    pinned = torch.from_numpy(data).pin_memory()
    hdata = pinned.numpy()

    def host_push():
        # a continuous stream: the recording is replayed from the start when it runs out (the
        # step's rows then go in as two pushes, both straight from the pinned recording)
        if pos[0] + chunk > hdata.shape[0]:
            s2.push(hdata[pos[0]:])
            pos[0] = pos[0] + chunk - hdata.shape[0]
            s2.push(hdata[: pos[0]])
        else:
            s2.push(hdata[pos[0]: pos[0] + chunk])
            pos[0] += chunk

    for _ in range(a.warmup + 1):
        host_push()
        s2.poll(out=obuf)
    drain(s2)
    barrier()
    torch.cuda.synchronize(dev)
    # a streaming caller keeps one group in flight: push step k (its host-to-device copy and
    # launches), then collect step k-1 (lss_poll waits for the oldest group only)
    n_sp = 0
    t_push = t_poll = 0.0
    t0 = time.perf_counter()
    for k in range(a.steps):
        ta = time.perf_counter()
        host_push()
        tb = time.perf_counter()
        if k > 0:
            n_sp += len(s2.poll(out=obuf))
        t_push += tb - ta
        t_poll += time.perf_counter() - tb
    n_sp += drain(s2)
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, world, f"cuda:{dev}")
    e2e = {"value": whole_job_rate(units, e2e_s, world), "unit": UNIT,
           "h2d_bytes_per_step": chunk * C * 2, "d2h_bytes_per_step": int(n_sp / a.steps * SPIKE_REC_BYTES),
           "path": "lss_push_batch + lss_poll from pinned host int16 rows, one group in flight",
           "host_ms_per_step": {"push": 1e3 * t_push / a.steps, "poll": 1e3 * t_poll / a.steps}}
    s2.close()

    # ---- per-batch latency (one batch per launch) --------------------------------------------
    latency = batch_latency(a.gemm_path, a.latency_batches, a.match_keep)

    # ---- the chosen path on eight concurrent probe streams (rank 0) ----------------------------
    chosen_block = None
    if rank == 0 and a.chosen_seconds > 0 and a.gemm_path == 0:
        chosen_block = run_chosen(a, dev)

    # ---- CPU baseline (rank 0) ----------------------------------------------------------------
    cpu = None
    if rank == 0 and not a.no_cpu:
        rate, times = cpu_oracle_rate(data, oss_dir, a.cpu_sample)
        cpu = {"value": rate, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"{a.cpu_sample} batches of 1500 new samples (+2*61) through the torch float32 form of the "
                         f"oracle (Kilosort filter + run_matching + xfeat + positions, the vendored path's torch "
                         f"operations), {os.cpu_count()} host threads, {sum(times):.1f} s"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded generator, shapes of the named config)",
                "config": workload_config(a, cfg, G), "e2e": e2e, "latency": latency, "roofline": roof,
                "cpu_baseline": cpu, "clocks": clk.summary(), "chosen_tier": tier, "chosen": chosen_block,
                "highpass_stateful": stateful,
                "gpu_launches": launches_per_step * a.steps,
                "spikes_per_batch": spikes_per_batch,
                "realtime_factor": value / (C * 30000.0)}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# -------------------------------------------------------------------------------------------
# threshold crossing
# -------------------------------------------------------------------------------------------
TC_METRIC = "ch*samples/s (threshold crossing, events identical to the reference's test)"
TC_CHANNELS, TC_THRESHOLD = 384, 3.0


def tc_dataset(rows: int):
    from livespikesorter_gb300 import synth
    data = synth.threshold_recording(2 * rows, TC_CHANNELS, seed=1)
    from oracle import tc_oracle  # calibration of the constants the detector is built with
    means, medians = tc_oracle.calibrate(data[:30000])
    return data, means, medians


def tc_config(a):
    return {"workload": f"threshold crossing, {TC_CHANNELS} ch x 30 kHz raw int16, pushes of {a.tc_rows} rows "
                        f"({a.tc_rows / 30000:.0f} s), threshold {TC_THRESHOLD} x per-channel median",
            "channels": TC_CHANNELS, "rows_per_push": a.tc_rows, "threshold_std": TC_THRESHOLD,
            "l2": "each push reads a fresh 461 MB slice (two slices alternate), larger than the 129 MB L2",
            "parallelism": "single"}


def tc_cpu_rate(data, means, medians, rows=30000, reps=3):
    from oracle import tc_oracle
    sample = data[:rows]
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        tc_oracle.threshold_crossings(sample, means, medians, TC_THRESHOLD)
        times.append(time.perf_counter() - t0)
    return rows * TC_CHANNELS / float(np.median(times)), times


def run_tc_reference(a):
    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    data, means, medians = tc_dataset(a.tc_rows)
    rows = min(a.tc_rows, 60000)
    times = []
    from oracle import tc_oracle
    for i in range(a.warmup + a.steps):
        t0 = time.perf_counter()
        tc_oracle.threshold_crossings(data[:rows], means, medians, TC_THRESHOLD)
        if i >= a.warmup:
            times.append(time.perf_counter() - t0)
    rate = rows * TC_CHANNELS / float(np.mean(times))
    line = {"metric": TC_METRIC, "value": rate, "unit": UNIT, "impl": "reference", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * float(np.mean(times)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int16",
            "data": "synthetic (seeded generator)", "config": tc_config(a),
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": f"{rows} rows x {TC_CHANNELS} ch per step through the numpy oracle"},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_tc_gpu(a):
    import torch
    from livespikesorter_gb300 import threshold
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    n = a.tc_rows
    C = TC_CHANNELS
    data, means, medians = tc_dataset(n)
    d_data = torch.from_numpy(data).to(f"cuda:{dev}")
    base = d_data.data_ptr()
    tc = threshold.ThresholdCrossing(means, medians, TC_THRESHOLD, device=dev, max_rows=n, profile=1)

    def step(i):
        tc.push_device(base + (i % 2) * n * C * 2, n, first_row_sample=(i % 2) * n)

    for i in range(a.warmup):
        step(i)
    ev_warm = tc.poll_all()
    t_base, k_base = tc.stage_times()
    torch.cuda.synchronize(dev)
    # each step: one push of device-resident rows, then its events read back through lss_tc_poll;
    # value = rows x channels / the device time of the push's kernels (CUDA events on the
    # detector's stream around count, offsets, emit and the copy to host memory); the wall time of
    # the same loop, host event reads included, is reported beside it
    n_events = 0
    with ClockSampler(dev) as clk:
        t0 = time.perf_counter()
        for i in range(a.steps):
            step(a.warmup + i)
            n_events += len(tc.poll(cap=n * C // 16))
        wall = time.perf_counter() - t0
    n_events += len(tc.poll_all())
    t_all, k_all = tc.stage_times()
    stage = {k: (t_all[k] - t_base[k]) / max(1, k_all - k_base) for k in t_all}
    ms = sum(stage[k] for k in ("count", "offsets", "emit", "d2h")) * a.steps
    launches = tc.kernel_launches() * a.steps
    value = a.steps * n * C / (ms / 1e3)
    hbm, _, src = peaks()
    count_bytes = 2.0 * n * C
    roof = {"kernel": "tc_count_kernel", "bound": "hbm", "achieved": count_bytes / 1e9 / (stage["count"] / 1e3),
            "peak": hbm, "unit": "GB/s", "peak_source": src, "traffic": None, "ms_per_launch": stage["count"],
            "stage_ms_per_launch": stage,
            "algorithmic_bytes_per_launch": count_bytes}
    roof["frac"] = roof["achieved"] / hbm
    tc.close()
    del d_data

    # end to end: pinned host rows -> lss_tc_push -> lss_tc_poll
    tc2 = threshold.ThresholdCrossing(means, medians, TC_THRESHOLD, device=dev, max_rows=n)
    hdata = torch.from_numpy(data).pin_memory().numpy()
    for i in range(a.warmup):
        tc2.push(hdata[(i % 2) * n:(i % 2 + 1) * n], (i % 2) * n)
    tc2.poll_all()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    n_ev2 = 0
    for i in range(a.steps):
        tc2.push(hdata[(i % 2) * n:(i % 2 + 1) * n], (i % 2) * n)
        n_ev2 += len(tc2.poll_all())
    e2e_s = time.perf_counter() - t0
    tc2.close()
    e2e = {"value": a.steps * n * C / e2e_s, "unit": UNIT, "h2d_bytes_per_step": n * C * 2,
           "d2h_bytes_per_step": int(16 * n_ev2 / a.steps),
           "path": "lss_tc_push + lss_tc_poll from pinned host int16 rows"}
    cpu = None
    if not a.no_cpu:
        rate, times = tc_cpu_rate(data, means, medians)
        cpu = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"30000 rows x {C} ch through the numpy oracle (float32 subtract, double compare, "
                         f"channel-major order), median of {len(times)}"}
    line = {"metric": TC_METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int16", "data": "synthetic (seeded generator)", "config": tc_config(a), "e2e": e2e,
            "roofline": roof, "cpu_baseline": cpu, "clocks": clk.summary(), "gpu_launches": launches,
            "events_per_push": n_events / a.steps, "warmup_events": len(ev_warm),
            "value_basis": "device time of the four kernels per push (CUDA events on the detector's stream)",
            "wall_ms_per_step_with_event_reads": 1e3 * wall / a.steps}
    print(json.dumps(line))
    return 0


# -------------------------------------------------------------------------------------------
# serving: concurrent probe streams
# -------------------------------------------------------------------------------------------
SERVING_STREAMS = [  # (channels, templates, batch samples)
    (384, 1000, 3000), (384, 500, 1500), (384, 250, 750), (192, 300, 1500),
    (192, 128, 3000), (96, 64, 750), (96, 100, 1500), (384, 700, 2250)]


def _serving_data(streams, seconds, seed0):
    from livespikesorter_gb300 import synth
    out = []
    for i, (C, T, NT) in enumerate(streams):
        cfg = synth.SynthConfig(n_chan=C, n_units=T, n_samples=int(seconds * 30000), drift_um=20.0,
                                seed=seed0 + i)
        d, data, _ = synth.cached_dataset(cfg)
        out.append((d, data, NT))
    return out


def _run_streams(sets, paced: bool, jitter: float = 0.2, seed: int = 0, gate=None, opts=None, spikes=None):
    """One thread per stream: push each batch (paced at 30 kHz with +/-jitter, or back to back),
    then poll its spikes; returns per-batch latencies (ms), wall seconds and new samples x channels.
    gate = (params, logit threshold, dilation) sets the learned proposal gate on every handle; opts =
    extra sorter parameters (gemm_path, match_keep); spikes = a list that receives each stream's
    spikes."""
    from livespikesorter_gb300 import sorter
    handles = [sorter.OnlineSorter(d, batch_samples=NT, max_iters=50, group_batches=1, **(opts or {}))
               for d, _, NT in sets]
    if gate is not None:
        for h in handles:
            h.set_proposal(*gate)
    for (d, data, NT), h in zip(sets, handles):   # warm-up: one window each
        h.push(data[:NT + 2 * 61], 0)
        h.poll_all()
    lat = [[] for _ in sets]
    work = [0] * len(sets)
    got = [[] for _ in sets]
    errors = []
    barrier = threading.Barrier(len(sets) + 1)

    def run(i):
        try:
            d, data, NT = sets[i]
            h = handles[i]
            rng = np.random.default_rng(seed + i)
            out = np.zeros(1 << 16, sorter.SPIKE_DTYPE)
            p = NT + 2 * 61
            barrier.wait()
            t_next = time.perf_counter()
            while p + NT <= data.shape[0]:
                if paced:
                    t_next += NT / 30000.0 * (1.0 + rng.uniform(-jitter, jitter))
                    dt = t_next - time.perf_counter()
                    if dt > 0:
                        time.sleep(dt)
                t1 = time.perf_counter()
                h.push(data[p:p + NT])
                r = h.poll(out=out)
                lat[i].append(1e3 * (time.perf_counter() - t1))
                if spikes is not None and len(r):
                    got[i].append(r.copy())
                work[i] += NT * data.shape[1]
                p += NT
        except Exception as e:
            errors.append(repr(e))

    th = [threading.Thread(target=run, args=(i,)) for i in range(len(sets))]
    for t in th:
        t.start()
    barrier.wait()
    t0 = time.perf_counter()
    for t in th:
        t.join()
    wall = time.perf_counter() - t0
    for h in handles:
        h.close()
    if errors:
        raise RuntimeError(errors[0])
    if spikes is not None:
        from livespikesorter_gb300 import sorter as _s
        spikes.extend(np.concatenate(g) if g else np.zeros(0, _s.SPIKE_DTYPE) for g in got)
    return lat, wall, work


# candidate paths of the chosen-path selection: (label, sorter parameters, arithmetic)
CHOSEN_CANDIDATES = [
    ("fp32", {"gemm_path": 0, "match_keep": 0}, "3xTF32 tcgen05 GEMMs (FP32-accurate), FP32 matching loop"),
    ("bf16x3", {"gemm_path": 3, "match_keep": 0},
     "bf16 splits (hi*hi + hi*lo + lo*hi on kind::f16), fp32 accumulate, FP32 matching loop"),
    ("bf16x3_keep16", {"gemm_path": 3, "match_keep": 16},
     "bf16 splits, matching loop on each sample's 16 templates of largest initial score"),
    ("bf16x3_keep24", {"gemm_path": 3, "match_keep": 24},
     "bf16 splits, matching loop on each sample's 24 templates of largest initial score"),
    ("bf16x3_keep16w24", {"gemm_path": 3, "match_keep": 16, "match_keep_wide": 24, "match_keep_crowd": 0.5},
     "bf16 splits, matching loop on each sample's 16 templates of largest initial score, 24 where the 16th "
     "largest initial Cf exceeds Th^2 / 2 (crowded samples)"),
    ("bf16x1_rescore", {"gemm_path": 4, "match_keep": 0},
     "one BF16 product (kind::f16), fp32 accumulate, accepted candidates re-scored in FP32"),
    ("fp8_rescore", {"gemm_path": 5, "match_keep": 0},
     "one FP8 e4m3 product (kind::f8f6f4) with per-(component, channel) and per-template scales, fp32 "
     "accumulate, accepted candidates re-scored in FP32"),
]


def run_chosen(a, dev):
    """The headline of the metric: the chosen precision path against plain FP32 on eight concurrent
    384-channel / 500-template probe streams of 1500-sample (50 ms) batches, one handle (CUDA stream)
    and host thread each -- the reference's one-sorter-per-probe model (src/main.cpp:77-85) on one
    GPU.  Every candidate path runs unpaced on the same eight streams (each stream pushes its next
    batch as soon as the last one's spikes are back): its aggregate throughput and its spike
    agreement with plain FP32 over every batch.  The chosen path is the fastest candidate at
    >= 99.5 % agreement with amplitudes within 1e-3 on >= 99.5 % of the matched spikes (plain FP32
    qualifies by definition); it then runs paced at 30 kHz (+/-20 % jitter) for per-batch
    push-to-spikes p50/p99."""
    streams = [(384, 500, NT)] * 8
    sets = _serving_data(streams, a.chosen_seconds, seed0=200)
    rt = 8 * 384 * 30000.0
    cands = [c for c in CHOSEN_CANDIDATES if a.chosen_only is None or c[0] in ("fp32", a.chosen_only)]
    runs = {}
    with ClockSampler(dev) as clk:
        for label, opts, _ in cands:
            sp = []
            lat, wall, work = _run_streams(sets, paced=False, opts=opts, spikes=sp)
            runs[label] = (lat, wall, work, sp)
        sp_f = runs["fp32"][3]
        table = []
        for label, opts, arith in cands:
            lat, wall, work, sp = runs[label]
            n_ref = n_m = n_amp = 0
            for f, c in zip(sp_f, sp):
                frac, amp_ok = spike_agreement(f, c)
                n_ref += len(f)
                n_m += frac * len(f)
                n_amp += amp_ok * frac * len(f)
            la = np.concatenate([np.asarray(x) for x in lat])
            rate = sum(work) / wall
            table.append({"label": label, "params": opts, "arithmetic": arith, "ch_samples_per_s": rate,
                          "realtime_factor": rate / rt, "spikes_per_s": sum(len(x) for x in sp) / wall,
                          "p50_ms": float(np.percentile(la, 50)), "p99_ms": float(np.percentile(la, 99)),
                          "matched_vs_fp32": n_m / max(n_ref, 1), "amp_within_1e-3": n_amp / max(n_m, 1e-9),
                          "spikes": int(sum(len(x) for x in sp)), "batches": int(la.size)})
        ok = [r for r in table if r["label"] == "fp32" or (r["matched_vs_fp32"] >= 0.995 and
                                                          r["amp_within_1e-3"] >= 0.995)]
        best = max(ok, key=lambda r: r["ch_samples_per_s"])
        lat_p, wall_p, work_p = _run_streams(sets, paced=True, opts=best["params"])
    lp = np.concatenate([np.asarray(x) for x in lat_p])
    plain = next(r for r in table if r["label"] == "fp32")
    return {"path": {**best["params"], "label": best["label"], "arithmetic": best["arithmetic"],
                     "proposal_gate": False},
            "streams": "8 x (384 ch, 500 templates, 1500-sample batches = 50 ms), one handle + host thread each",
            "rule": "fastest unpaced candidate at >= 99.5 % spike agreement with plain FP32 and >= 99.5 % of "
                    "amplitudes within 1e-3",
            "paced": {"p50_ms": float(np.percentile(lp, 50)), "p99_ms": float(np.percentile(lp, 99)),
                      "max_ms": float(lp.max()), "batches": int(lp.size), "batch_ms_of_signal": 1e3 * NT / 30000.0,
                      "pacing": "30 kHz, +/-20 % jitter per batch"},
            "unpaced": {k: best[k] for k in ("ch_samples_per_s", "realtime_factor", "spikes_per_s", "p50_ms",
                                             "p99_ms")},
            "plain_fp32_unpaced": {k: plain[k] for k in ("ch_samples_per_s", "realtime_factor", "spikes_per_s",
                                                         "p50_ms", "p99_ms")},
            "speedup_vs_plain_fp32": best["ch_samples_per_s"] / plain["ch_samples_per_s"],
            "agreement_vs_plain_fp32": {"batches": best["batches"], "spikes_fp32": plain["spikes"],
                                        "spikes_chosen": best["spikes"], "matched": best["matched_vs_fp32"],
                                        "amp_within_1e-3": best["amp_within_1e-3"],
                                        "rule": "same template, |dt| <= 1 sample, amplitude within 1e-3 relative"},
            "candidates": table,
            "targets": {"realtime_factor": 10.0, "p99_ms": 5.0, "agreement": 0.995},
            "clocks": clk.summary()}


def run_serving(a):
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    t_start = time.perf_counter()
    sets = _serving_data(SERVING_STREAMS, a.serving_seconds, seed0=100)
    with ClockSampler(dev) as clk:
        lat, wall, work = _run_streams(sets, paced=True)
    all_lat = np.concatenate([np.asarray(x) for x in lat])
    per_stream = [{"channels": C, "templates": T, "batch_samples": NT, "batches": len(l),
                   "p50_ms": float(np.percentile(l, 50)), "p99_ms": float(np.percentile(l, 99)),
                   "batch_ms_of_signal": 1e3 * NT / 30000.0}
                  for (C, T, NT), l in zip(SERVING_STREAMS, lat)]
    paced = {"p50_ms": float(np.percentile(all_lat, 50)), "p99_ms": float(np.percentile(all_lat, 99)),
             "max_ms": float(all_lat.max()), "batches": int(all_lat.size),
             "ch_samples_per_s": sum(work) / wall, "wall_s": wall, "streams": per_stream}
    lat_u, wall_u, work_u = _run_streams(sets, paced=False)
    lu = np.concatenate([np.asarray(x) for x in lat_u])
    unpaced = {"ch_samples_per_s": sum(work_u) / wall_u, "realtime_factor": (sum(work_u) / wall_u) /
               (30000.0 * sum(C for C, _, _ in SERVING_STREAMS)), "p50_ms": float(np.percentile(lu, 50)),
               "p99_ms": float(np.percentile(lu, 99)), "wall_s": wall_u}
    sets8 = _serving_data([(384, 500, 1500)] * 8, a.serving_seconds, seed0=200)
    lat8, wall8, work8 = _run_streams(sets8, paced=False)
    l8 = np.concatenate([np.asarray(x) for x in lat8])
    eight = {"ch_samples_per_s": sum(work8) / wall8, "realtime_factor": (sum(work8) / wall8) / (8 * 384 * 30000.0),
             "p50_ms": float(np.percentile(l8, 50)), "p99_ms": float(np.percentile(l8, 99)), "wall_s": wall8}
    line = {"metric": "serving: p99 push-to-spikes latency per batch, 8 concurrent streams at 30 kHz pacing",
            "value": paced["p99_ms"], "unit": "ms", "n_gpus": 1, "steps": int(all_lat.size), "warmup": 1,
            "ms_per_step": paced["p50_ms"], "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded generator, shapes of the serving config)",
            "config": {"workload": "8 probe streams (96/192/384 ch, 64-1000 templates, 750-3000-sample "
                                   "batches), 30 kHz pacing +/-20 % jitter, one handle + host thread each",
                       "streams": [list(x) for x in SERVING_STREAMS], "seconds_per_stream": a.serving_seconds,
                       "parallelism": "single GPU, 8 CUDA streams"},
            "paced": paced, "unpaced": unpaced, "eight_384ch_unpaced": eight, "clocks": clk.summary(),
            "wall_s": time.perf_counter() - t_start}
    print(json.dumps(line))
    return 0


def run_proposal(a):
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    from livespikesorter_gb300 import proposal, sorter, synth
    t_start = time.perf_counter()
    cfg = synth.config_stream(seconds=a.seconds, seed=1)
    oss_dir, data, rec = synth.cached_dataset(cfg)
    C, nt = cfg.n_chan, cfg.nt
    W = NT + 2 * nt
    oss_Wall3 = np.load(Path(oss_dir) / "Wall3.npy")
    starts = proposal.neighbourhoods(C)
    owner = proposal.template_owner(oss_Wall3)
    nw = min(a.prop_train_windows, (data.shape[0] - 2 * nt) // NT)
    G = a.group
    with sorter.OnlineSorter(oss_dir, device=dev, batch_samples=NT, max_iters=50, group_batches=G) as s:
        wins = proposal.batch_windows(data, 0, nw, NT, nt)
        labels, _ = proposal.plain_labels(s, wins, owner, len(starts))
        z = proposal.whitened(s, wins)
    with proposal.ProposalTrainer(W, nt, max_examples=64, seed=0) as tr:
        tr.step(z, proposal.all_pairs(1, starts)[:64], labels[0].reshape(-1, labels.shape[-1])[:64])  # warm-up
        tr.params = proposal.init_params(0)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        losses = proposal.train(tr, z, labels, starts, steps=a.prop_steps, batch=64, seed=0)
        train_s = time.perf_counter() - t0
        zw = proposal.window_logits(tr, z, starts)
        params = tr.params
    del z
    thr = proposal.choose_threshold(zw, labels, 1, 0.999)   # 99.9 % of training cells: held-out recall >= 99.5 %
    step_flop = 3 * 2 * 64 * W * 7 * sum(o * i for o, i in proposal.SHAPES)   # forward + two backward passes
    held = {}
    rate_gated = rate_plain = None
    for rate, seed in ((5.0, 301), (10.0, 302), (20.0, 303), (40.0, 304)):
        r = synth.rerecord(rec, seed, rate_hz=rate, n_samples=G * NT + 2 * nt)
        hw = proposal.batch_windows(r.data, 0, G, NT, nt)
        with sorter.OnlineSorter(oss_dir, device=dev, batch_samples=NT, max_iters=50, group_batches=G,
                                 profile=1) as s:
            plain = np.concatenate(s.sort_windows(hw))
            s.set_proposal(params, logit_threshold=thr, dilate=1)
            gated = np.concatenate(s.sort_windows(hw))
            cells, opened = s.proposal_stats()
            if rate == 10.0:
                d_rows = torch.from_numpy(r.data).to(f"cuda:{dev}")
                ext = torch.cuda.ExternalStream(s.cuda_stream(), device=f"cuda:{dev}")

                ctr = [0]

                def push():
                    # the same G windows again, as a continuing stream
                    s.push_device_span(d_rows.data_ptr(), G, ctr[0] * G * NT)
                    ctr[0] += 1

                def dev_ms(reps=5):
                    for _ in range(2):
                        push()
                    s.poll_all()
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    with torch.cuda.stream(ext):
                        e0.record(ext)
                    for i in range(reps):
                        push()
                    with torch.cuda.stream(ext):
                        e1.record(ext)
                    e1.synchronize()
                    s.poll_all()
                    return e0.elapsed_time(e1) / reps

                ms_g = dev_ms()
                s.set_proposal(None)
                ms_p = dev_ms()
                rate_gated = G * NT * C / (ms_g / 1e3)
                rate_plain = G * NT * C / (ms_p / 1e3)
                del d_rows
        recall, amp_ok = spike_agreement(plain, gated)
        held[f"{rate:g}Hz"] = {"spikes_plain": int(len(plain)), "spikes_gated": int(len(gated)),
                               "recall": recall, "amp_within_1e-3": amp_ok, "cells_open_frac": opened / max(1, cells)}
    # eight 384-channel streams at once, every handle gated (held-out seeds, 10 Hz)
    secs = min(a.serving_seconds, 4.0)
    sets = [(oss_dir, synth.rerecord(rec, 500 + i, rate_hz=10.0, n_samples=int(secs * 30000)).data, NT)
            for i in range(8)]
    gate = (params, thr, 1)
    lat_p, wall_p, work_p = _run_streams(sets, paced=True, gate=gate)
    lat_u, wall_u, work_u = _run_streams(sets, paced=False, gate=gate)
    lp, lu = np.concatenate([np.asarray(x) for x in lat_p]), np.concatenate([np.asarray(x) for x in lat_u])
    eight = {"paced_p50_ms": float(np.percentile(lp, 50)), "paced_p99_ms": float(np.percentile(lp, 99)),
             "paced_batches": int(lp.size), "unpaced_ch_samples_per_s": sum(work_u) / wall_u,
             "unpaced_realtime_factor": (sum(work_u) / wall_u) / (8 * C * 30000.0),
             "unpaced_p99_ms": float(np.percentile(lu, 99)), "seconds_per_stream": secs,
             "batch_ms_of_signal": 1e3 * NT / 30000.0}
    line = {"metric": "proposal gate: recall of the plain matcher's spikes and cells closed, 384 ch / 500 templates",
            "value": min(h["recall"] for h in held.values()), "unit": "recall (min over firing rates)",
            "n_gpus": 1, "steps": a.prop_steps, "warmup": 1, "ms_per_step": 1e3 * train_s / a.prop_steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 train, bf16 weights gate",
            "data": "synthetic (seeded generator; held-out seeds of the same units)",
            "config": {"workload": "4-layer channel-local conv net (16 ch neighbourhoods, 64 hidden, 7 taps), "
                                   "32-sample windows, dilation 1, threshold for 0.995 cell recall on the training "
                                   "windows", "train_windows": nw, "batch_examples": 64, "adam_lr": 1e-3,
                       "neighbourhoods": int(len(starts)), "logit_threshold": thr},
            "training": {"steps": a.prop_steps, "s": train_s, "loss_first20": float(losses[:20].mean()),
                         "loss_last20": float(losses[-20:].mean()),
                         "tflops": step_flop * a.prop_steps / train_s / 1e12,
                         "label_positive_frac": float(labels.mean())},
            "held_out": held,
            "throughput_10Hz": {"gated": rate_gated, "plain": rate_plain, "unit": UNIT,
                                "group_batches": G},
            "eight_384ch_streams_gated": eight,
            "wall_s": time.perf_counter() - t_start}
    print(json.dumps(line))
    return 0


def main():
    a = args_()
    if a.serving:
        return run_serving(a)
    if a.path == "proposal":
        return run_proposal(a)
    if a.path == "tc":
        return run_tc_reference(a) if a.impl == "reference" else run_tc_gpu(a)
    if a.impl == "reference":
        return run_reference(a)
    return run_gpu(a)


if __name__ == "__main__":
    sys.exit(main())
