#!/usr/bin/env python3
"""Golden vectors for the randomized branching fuzz (tests/test_fuzz.py).

Runs the reference's own fuzz case builder and its rollback-Fenwick "rf" arm,
compiled from the reference sources by ``make -f oracle/ref.mk fuzz STATES=n``
(harness oracle/ref_fuzz.cpp), and records per case the parameters, the SHA-256
of the fixture file the reference wrote and the SHA-256 of its answer vector.
Two state counts: 33 (the reference fuzz's own build, fuzz_fullpath.cpp:23-26)
and 257 (deeper trees, several state blocks on the GPU).

Usage: python tests/golden/make_fuzz_golden.py [--ref <reference checkout>]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
RUNS = [(33, 600), (257, 150)]   # (states, cases)


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference checkout (default: $BW_REFERENCE_DIR, else a "
                    "'reference' directory beside this repository)")
    args = ap.parse_args()
    if args.ref is None:
        import sys
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle  # noqa: E402  (test infrastructure)
        ref = oracle.reference_dir()
        if ref is None:
            raise SystemExit("reference checkout not found: pass --ref or set BW_REFERENCE_DIR")
        args.ref = str(ref)
    out = {"source": "reference fuzz_fullpath.cpp build_case + rf arm (oracle/ref_fuzz.cpp)", "runs": []}
    with tempfile.TemporaryDirectory() as tmp:
        for states, n in RUNS:
            subprocess.run(["make", "-s", "-f", "oracle/ref.mk", f"REF={args.ref}", f"STATES={states}", "fuzz"],
                           cwd=ROOT, check=True)
            p = subprocess.run([str(ROOT / "oracle" / "_ref" / f"fuzz_ref_{states}"), "--cases", str(n),
                                "--fixture", str(Path(tmp) / "fx.bin")], capture_output=True, text=True,
                               check=True)
            cases = [json.loads(line) for line in p.stdout.splitlines() if line.strip()]
            assert len(cases) == n
            out["runs"].append({"states": states, "cases": cases})
            print(f"states {states}: {n} cases")
    (HERE / "fuzz_golden.json").write_text(json.dumps(out, separators=(",", ":")) + "\n")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
