"""Build the oracle's reference-backed checkers into oracle/_ref/ -- TEST INFRASTRUCTURE ONLY.

``payload_ref``: oracle/payload_ref.cpp compiled against the reference's vendored cereal headers
(External/cereal, header-only) where they lie in the reference checkout.  Nothing else of the
reference is compiled.  Without the checkout (the reference is absent) nothing is built and the
committed golden bytes in tests/golden/ stand in for it.
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


def build(verbose: bool = False):
    """Returns the path of payload_ref, or None when the reference checkout is absent."""
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
