"""Check oss_input/ directories without a GPU: ``python -m livespikesorter_gb300.validate DIR [DIR ...]``.

Runs the sorter's own loader and shape checks (``lss_validate_oss_input``) -- the checks
``lss_open`` makes before it touches a device -- and prints each directory's dimensions or the
reason it would be refused.  Exit status 0 when every directory passes, 1 otherwise.
"""
from __future__ import annotations

import argparse
import sys

from .sorter import STATUS, SorterError, validate_oss_input


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m livespikesorter_gb300.validate", description=__doc__.splitlines()[0])
    ap.add_argument("dirs", nargs="+", help="oss_input/ directories")
    a = ap.parse_args(argv)
    bad = 0
    for d in a.dirs:
        try:
            i = validate_oss_input(d)
        except SorterError as e:
            bad += 1
            print(f"{d}: REFUSED ({STATUS.get(e.status, e.status)}) {e}")
            continue
        print(f"{d}: OK  channels {i.C}, templates {i.T} (final {i.T_final}), PCs {i.K}, nt {i.nt}, "
              f"nearest channels {i.nC}, nt0min {i.nt0min}, Th {i.th:g}, duplicate bins {i.dup_bins}")
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main())
