"""Golden bytes of the per-batch spike message, written by the reference's own cereal.

Builds oracle/_ref/payload_ref (oracle/build_ref.py: oracle/payload_ref.cpp against the
reference's vendored External/cereal headers), serializes a few seeded messages with both `long`
widths and saves inputs and bytes to tests/golden/payload_cereal.npz.  Run from the repository
root with the reference checkout present:  python tests/golden/make_payload_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import build_ref  # noqa: E402
from oracle import payload_oracle as po  # noqa: E402


def cases():
    rng = np.random.default_rng(2024)
    out = []
    for n in (0, 1, 7, 230):
        times = np.sort(rng.integers(0, 2_000_000_000, n)).astype(np.int64)
        templates = rng.integers(-1, 500, n).astype(np.int64)
        amps = rng.lognormal(3.0, 0.5, n).astype(np.float32)
        hdr = {"recording_offset": int(rng.integers(0, 10**9)), "stream_sample_ct": int(rng.integers(0, 10**10)),
               "vrms": 0.0, "p2p": float(np.float32(rng.uniform(50, 900))),
               "process_time": int(rng.integers(0, 10**7)), "event_stream_sample_ct": 0,
               "predict_label": 0, "label": 0, "n_trials": 0, "n_correct": 0, "confidence": 0.0}
        if n == 7:   # the decoder-side fields set too, and values past 32 bits
            hdr.update(event_stream_sample_ct=-5, predict_label=3, label=-2, n_trials=41, n_correct=17,
                       confidence=0.8125, vrms=12.5, stream_sample_ct=(1 << 33) + 12345)
            times[-1] = (1 << 32) + 7
        out.append((hdr, times, templates, amps))
    return out


def main():
    exe = build_ref.build(verbose=True)
    if exe is None:
        raise SystemExit("the reference checkout (External/cereal) is needed to make these fixtures")
    arrays = {}
    for i, (hdr, times, templates, amps) in enumerate(cases()):
        arrays[f"c{i}_times"], arrays[f"c{i}_templates"], arrays[f"c{i}_amps"] = times, templates, amps
        arrays[f"c{i}_header"] = np.array([hdr[k] for k in po.HEADER], dtype=np.float64)
        for lb in (4, 8):
            b = po.cereal_serialize(exe, hdr, times, templates, amps, lb)
            arrays[f"c{i}_bytes{lb}"] = np.frombuffer(b, np.uint8)
    out = ROOT / "tests" / "golden" / "payload_cereal.npz"
    np.savez_compressed(out, n_cases=len(cases()), **arrays)
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
