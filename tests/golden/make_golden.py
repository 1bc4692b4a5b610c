#!/usr/bin/env python3
"""Generate the golden fixtures and answer hashes used by the parity tests.

Fixtures follow the reference's synthetic BWBASE02 generator
(tools/prep_scale_workloads.py:32-63): numpy ``default_rng(seed)``; uniform
timestamps over [0, span); uniform groups; amounts ``lognormal(5, 1) * 100``
truncated to int64 plus 1; all factors 1000; labels 0..G-1; header t_min = 0,
t_max = span - 1, amount_scale 2.  The bytes are pinned by the fixture SHA-256
values the reference tool prints for the same arguments.

Golden answer hashes come from three sources, recorded per case:
* ``published``: SHA-256 values stored in the reference's results tree
  (results/general_router_final2_20261102/summary.json, cells 1d_q2 and 1d_q8);
* ``reference``: the reference's own ``oracle`` binary built from source by
  oracle/ref.mk (only where the reference sources are mounted);
* ``oracle``: this repository's C restatement (oracle/bw_oracle.c).

Usage: python tests/golden/make_golden.py [--ref-dir oracle/_ref]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import struct
import subprocess
import sys
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent

HDR = struct.Struct("<8s q i i q q q q q")
ROW = np.dtype([("t", "<i8"), ("a", "<i8"), ("g", "<i4"), ("p", "<i4")])

# (name, rows, groups, seed, span, fixture sha256 printed by the reference tool)
FIXTURES = {
    "check": (2000, 4, 20261131, 86_400_000_000,
              "a09bbbfcce53e1e25d70ecb3c6d460bd53cf7dfe168474e36c0ccccd9f3bd576"),
    "real3_100k": (100_000, 64, 20261151, 86_400_000_000,
                   "541e4908077fbeb0abadcc6a8919ffb2e9459b45c1dbb77da138eb19ea1b4f1f"),
    "survey_100k": (100_000, 64, 20261029, 86_400_000_000,
                    "4db7a8e6d7c7ed9db19b488829cfa7151aee7dfa7fc2b654efb1f86af8a8e702"),
}

# Reference-native golden cases: (fixture, states, topology, seed, factor period, q,
# published sha256 or None).  Ranges are per_state (BWH_RANGE_SCOPE=per_state).
CASES = [
    ("real3_100k", 2049, 0, 20261291, 59, 2,
     "4dd03937cd1e597ef99c14c74deb02cb351edf449e7adf86d187ce8434cec8ba"),
    ("real3_100k", 2049, 0, 20261292, 59, 8,
     "2af9e1493928ddb61025c5f08bb5793902fab6ea778b9f3a81598c8a48a19674"),
] + [("check", 2049, topo, 7, fp, 2, None) for topo in (0, 1, 2) for fp in (4, 37)] + [
    ("check", 2049, topo, 11, 4, 8, None) for topo in (0, 1, 2)]

# Shared-range cases (BWH_RANGE_SCOPE unset: one set of q nested ranges for every
# state, common.hpp:296-306), pinned by the reference oracle run without the
# per_state scope.
SHARED_CASES = [("check", 2049, topo, 7, 37, 2, None) for topo in (0, 1, 2)] + [
    ("check", 2049, 0, 11, 4, 8, None), ("real3_100k", 2049, 1, 20261291, 59, 4, None)]


# Large reference-native cases, too slow for the direct-scan oracle (about five
# minutes each); pinned by the reference's own v7 worker (panel_batch_v7fix.cpp,
# "compiled") built from source at the matching state count.
LARGE_CASES = [("survey_100k", 300_000, 0, 7, 37, 2)]


def make_fixture(rows: int, groups: int, seed: int, span: int) -> bytes:
    rng = np.random.default_rng(seed)
    ts = rng.integers(0, span, size=rows, dtype=np.int64)
    grp = rng.integers(0, groups, size=rows, dtype=np.int32)
    amount = (rng.lognormal(mean=5.0, sigma=1.0, size=rows) * 100).astype(np.int64) + 1
    rec = np.empty(rows, dtype=ROW)
    rec["t"], rec["a"], rec["g"], rec["p"] = ts, amount, grp, 0
    head = HDR.pack(b"BWBASE02", rows, groups, 0, rows, 0, 0, span - 1, 2)
    return (head + rec.tobytes() + np.full(groups, 1000, dtype="<i8").tobytes()
            + np.arange(groups, dtype="<i4").tobytes())


def fixture_bytes(name: str) -> bytes:
    """Fixture image: the committed compressed copy (bit-exact on every machine)."""
    return zlib.decompress((HERE / f"{name}.bin.z").read_bytes())


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-dir", default=str(ROOT / "oracle" / "_ref"))
    args = ap.parse_args()
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle  # noqa: E402  (test infrastructure)

    for name, (rows, groups, seed, span, want) in FIXTURES.items():
        img = make_fixture(rows, groups, seed, span)
        got = hashlib.sha256(img).hexdigest()
        if got != want:
            raise SystemExit(f"fixture {name}: sha {got} != reference tool {want}")
        (HERE / f"{name}.bin.z").write_bytes(zlib.compress(img, 9))
    out = {"fixtures": {k: v[4] for k, v in FIXTURES.items()}, "cases": []}
    for (fx_name, states, topo, seed, fp, q, published), per_state in (
            [(c, True) for c in CASES] + [(c, False) for c in SHARED_CASES]):
        img = fixture_bytes(fx_name)
        ans = oracle.direct_scan(oracle.Fixture(img), states, topo, seed, fp, q, per_state)
        sha = oracle.sha256_hex(ans.tobytes())
        rec = {"fixture": fx_name, "states": states, "topology": topo, "seed": seed,
               "factor_period": fp, "q": q, "per_state": per_state, "oracle": sha,
               "fnv1a": f"{oracle.fnv1a(ans.tobytes()):016x}", "n_answers": int(ans.size)}
        if published:
            rec["published"] = published
        ref = Path(args.ref_dir) / f"oracle_{states}"
        if ref.exists():
            tmp = ROOT / "_work" / "golden_fixture.bin"
            tmp.parent.mkdir(exist_ok=True)
            tmp.write_bytes(img)
            env = {k: v for k, v in os.environ.items() if k != "BWH_RANGE_SCOPE"}
            if per_state:
                env["BWH_RANGE_SCOPE"] = "per_state"
            p = subprocess.run([str(ref), "--fixture", str(tmp), "--topology", str(topo),
                                "--seed", str(seed), "--factor-period", str(fp), "--q", str(q),
                                "--out", str(tmp) + ".ans"], capture_output=True, text=True,
                               env=env, check=True)
            rec["reference"] = json.loads(p.stdout.strip().splitlines()[-1])["answers_sha256"]
        agree = {rec[k] for k in ("oracle", "published", "reference") if k in rec}
        if len(agree) != 1:
            raise SystemExit(f"golden disagreement: {rec}")
        out["cases"].append(rec)
        print(json.dumps(rec))
    out["large_cases"] = []
    old = {}
    if (HERE / "golden.json").exists():
        for r in json.loads((HERE / "golden.json").read_text()).get("large_cases", []):
            old[(r["fixture"], r["states"], r["topology"], r["seed"], r["factor_period"], r["q"])] = r
    for fx_name, states, topo, seed, fp, q in LARGE_CASES:
        key = (fx_name, states, topo, seed, fp, q)
        rec = dict(old.get(key, {}), fixture=fx_name, states=states, topology=topo, seed=seed,
                   factor_period=fp, q=q, per_state=True, n_answers=(states - 1) * q)
        ref = Path(args.ref_dir) / f"compiled_{states}"
        if ref.exists():
            tmp = ROOT / "_work" / "golden_fixture.bin"
            tmp.write_bytes(fixture_bytes(fx_name))
            env = dict(os.environ, BWH_RANGE_SCOPE="per_state")
            subprocess.run([str(ref), "--fixture", str(tmp), "--base-id", fx_name, "--topology",
                            str(topo), "--seed", str(seed), "--factor-period", str(fp), "--q",
                            str(q), "--answers", str(tmp) + ".ans", "--json", str(tmp) + ".json"],
                           capture_output=True, text=True, env=env, check=True)
            rec["reference"] = json.loads(Path(str(tmp) + ".json").read_text())["answers_sha256"]
        if "reference" not in rec:
            raise SystemExit(f"large case {key} has no reference hash (build oracle/ref.mk)")
        out["large_cases"].append(rec)
        print(json.dumps(rec))
    (HERE / "golden.json").write_text(json.dumps(out, indent=1) + "\n")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
