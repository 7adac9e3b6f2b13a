"""Helpers shared by the parity tests: spike-set matching and oss_input dirs from fixtures."""
from __future__ import annotations

from pathlib import Path

import numpy as np

from livespikesorter_gb300 import synth


def match_spikes(t_ref, k_ref, t_got, k_got, tol: int = 1):
    """Greedy one-to-one matching: same template, |dt| <= tol, exact-time pairs first.
    Returns index arrays (ref_idx, got_idx) of the matched pairs."""
    t_ref, k_ref = np.asarray(t_ref, np.int64), np.asarray(k_ref, np.int64)
    t_got, k_got = np.asarray(t_got, np.int64), np.asarray(k_got, np.int64)
    pool = {}
    for j in range(len(t_got)):
        pool.setdefault((int(k_got[j]), int(t_got[j])), []).append(j)
    used_r = np.zeros(len(t_ref), bool)
    ri, gi = [], []
    for dt in range(0, tol + 1):
        for i in range(len(t_ref)):
            if used_r[i]:
                continue
            k, t = int(k_ref[i]), int(t_ref[i])
            for cand in ((t,) if dt == 0 else (t - dt, t + dt)):
                lst = pool.get((k, cand))
                if lst:
                    gi.append(lst.pop(0))
                    ri.append(i)
                    used_r[i] = True
                    break
    return np.array(ri, np.int64), np.array(gi, np.int64)


def agreement(t_ref, k_ref, a_ref, t_got, k_got, a_got, tol: int = 1):
    """(fraction matched over the larger set, fraction of matched pairs with amplitude within
    1e-3 relative, max relative amplitude error)"""
    ri, gi = match_spikes(t_ref, k_ref, t_got, k_got, tol)
    if len(t_ref) == 0 and len(t_got) == 0:
        return 1.0, 1.0, 0.0
    denom = max(len(t_ref), len(t_got), 1)
    if len(ri) == 0:
        return len(ri) / denom, 1.0 if denom == 1 else 0.0, 0.0
    rel = np.abs(np.asarray(a_got)[gi] - np.asarray(a_ref)[ri]) / np.maximum(np.abs(np.asarray(a_ref)[ri]), 1e-12)
    return len(ri) / denom, float((rel <= 1e-3).mean()), float(rel.max())


def write_oss_from_arrays(z, out_dir) -> Path:
    """An oss_input/ dir from a fixture holding the exported arrays (tests/golden/*.npz)."""
    misc = np.asarray(z["misc"])
    T, K, C = z["Wall3"].shape
    oss = synth.OssInput(
        templates=z["pre_wf"], Wall3=z["Wall3"], ctc=z["ctc"], wPCA=z["wPCA"], pre_wf=z["pre_wf"],
        whitening=z["whitening"], drift=z["drift"], iCC=z["iCC"], iU=z["iU"], Ucc=z["Ucc"],
        hp_filter=z["hp_filter"], xc=z["xc"], yc=z["yc"], channel_map=np.arange(C, dtype=np.int32),
        template_map=np.arange(T, dtype=np.int32), centroids=z["centroids"],
        centroids_pca=np.zeros((T, K), np.float32), spike_templates=np.zeros(1, np.int64),
        misc={"nt0min": int(misc[0]), "numNearestChans": int(misc[1]), "Th_learned": float(misc[2]),
              "duplicate_spike_bins": int(misc[3])})
    return synth.write_oss_input(oss, out_dir)


def make_dataset(cfg: synth.SynthConfig, out_dir):
    """(oss_dir, int16 data [N, C], OssInput) for a seeded config, written under out_dir."""
    rec = synth.make_recording(cfg)
    oss = synth.build_oss_input(rec)
    d = synth.write_oss_input(oss, Path(out_dir) / "oss_input")
    return d, rec.data, oss
