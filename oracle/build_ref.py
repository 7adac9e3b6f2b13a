"""Build the oracle's reference-backed checkers into oracle/_ref/ -- TEST INFRASTRUCTURE ONLY.

``payload_ref``: oracle/payload_ref.cpp compiled against the reference's vendored cereal headers
(External/cereal, header-only) where they lie in the reference checkout.
``tc_ref``: the reference's src/SpikeSorter/ThresholdCrossing.cpp compiled unmodified where it
lies, with oracle/tc_ref_stubs.h force-included in place of its Windows / SpikeGLX / networking
headers, linked with oracle/tc_ref_driver.cpp (a scripted replay of int16 rows); it produces the
threshold-crossing fixture tests/golden/tc_reference.npz (tests/golden/make_tc_golden.py).
Without the checkout nothing is built and the committed golden files stand in for them.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
# the reference checkout: LSS_REFERENCE_DIR, else a "reference" directory beside this repository
REFERENCE = Path(os.environ.get("LSS_REFERENCE_DIR") or (HERE.parent.parent / "reference"))


def build_tc(verbose: bool = False):
    """Returns the path of tc_ref, or None when the reference checkout is absent."""
    src = REFERENCE / "src" / "SpikeSorter" / "ThresholdCrossing.cpp"
    cxx = shutil.which("g++") or shutil.which("c++")
    if not src.exists() or cxx is None:
        return None
    OUT.mkdir(exist_ok=True)
    exe = OUT / "tc_ref"
    deps = [HERE / "tc_ref_stubs.h", HERE / "tc_ref_driver.cpp"]
    if not exe.exists() or exe.stat().st_mtime < max(d.stat().st_mtime for d in deps):
        subprocess.run([cxx, "-std=c++17", "-O1", "-include", str(HERE / "tc_ref_stubs.h"), "-I", str(src.parent),
                        str(src), str(HERE / "tc_ref_driver.cpp"), "-o", str(exe), "-lpthread"], check=True)
    if verbose:
        print(f"built {exe}")
    return exe


def build(verbose: bool = False):
    """Returns the path of payload_ref, or None when the reference checkout is absent (tc_ref is
    built beside it)."""
    build_tc(verbose)
    inc = REFERENCE / "External"
    if not (inc / "cereal" / "archives" / "binary.hpp").exists():
        return None
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        return None
    OUT.mkdir(exist_ok=True)
    exe = OUT / "payload_ref"
    src = HERE / "payload_ref.cpp"
    if not exe.exists() or exe.stat().st_mtime < src.stat().st_mtime:
        subprocess.run([cxx, "-std=c++17", "-O1", "-isystem", str(inc), str(src), "-o", str(exe)], check=True)
    if verbose:
        print(f"built {exe}")
    return exe


if __name__ == "__main__":
    build(verbose=True)
