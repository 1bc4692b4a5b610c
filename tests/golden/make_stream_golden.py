#!/usr/bin/env python3
"""Golden BWLEV001 event streams for tests/test_stream.py.

Runs the reference's own stream emitter (emit_events.cpp, built unmodified from the
reference sources by ``make -f oracle/ref.mk emit STATES=2049``) on the committed
``check`` fixture for reference-native cases whose answer SHA-256 golden.json
already pins (published value, else the reference oracle's, else this
repository's oracle).  The emitter builds per-state ranges, so only per_state
cases qualify.  Writes the zlib-compressed streams (stream_*.bwlev.z) and
stream_golden.json (case parameters, record count, stream SHA-256, answer SHA-256).

Usage: python tests/golden/make_stream_golden.py [--ref <reference checkout>]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import subprocess
import sys
import tempfile
import zlib
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
STATES = 2049
CASES = [(0, 7, 4, 2), (1, 7, 4, 2), (2, 7, 4, 2), (0, 11, 4, 8)]   # topology, seed, factor period, q


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference checkout (default: $BW_REFERENCE_DIR, else a "
                    "'reference' directory beside this repository)")
    args = ap.parse_args()
    if args.ref is None:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle  # noqa: E402  (test infrastructure)
        ref = oracle.reference_dir()
        if ref is None:
            raise SystemExit("reference checkout not found: pass --ref or set BW_REFERENCE_DIR")
        args.ref = str(ref)
    subprocess.run(["make", "-s", "-f", "oracle/ref.mk", f"REF={args.ref}", f"STATES={STATES}", "emit"],
                   cwd=ROOT, check=True)
    emit = ROOT / "oracle" / "_ref" / f"emit_events_{STATES}"
    gold = json.loads((HERE / "golden.json").read_text())
    out = {"source": "reference emit_events.cpp on the check fixture", "states": STATES, "cases": []}
    with tempfile.TemporaryDirectory() as tmp:
        fx = Path(tmp) / "check.bin"
        fx.write_bytes(zlib.decompress((HERE / "check.bin.z").read_bytes()))
        for topo, seed, fp, q in CASES:
            want = [c for c in gold["cases"] if c["fixture"] == "check" and c["states"] == STATES and
                    c["topology"] == topo and c["seed"] == seed and c["factor_period"] == fp and c["q"] == q
                    and c["per_state"]]
            assert len(want) == 1, (topo, seed, fp, q)
            c = want[0]
            sha = c.get("published") or c.get("reference") or c["oracle"]
            path = Path(tmp) / "s.bwlev"
            p = subprocess.run([str(emit), "--fixture", str(fx), "--out", str(path), "--topology", str(topo),
                                "--seed", str(seed), "--factor-period", str(fp), "--q", str(q)],
                               capture_output=True, text=True, check=True)
            data = path.read_bytes()
            name = f"stream_t{topo}_s{seed}_f{fp}_q{q}.bwlev.z"
            (HERE / name).write_bytes(zlib.compress(data, 9))
            out["cases"].append({"file": name, "topology": topo, "seed": seed, "factor_period": fp, "q": q,
                                 "records": int(p.stdout.split("=")[1]), "stream_sha256":
                                 hashlib.sha256(data).hexdigest(), "answers_sha256": sha,
                                 "n_answers": c["n_answers"], "fnv1a": c["fnv1a"]})
            print(name, len(data), "bytes")
    (HERE / "stream_golden.json").write_text(json.dumps(out, indent=1) + "\n")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
