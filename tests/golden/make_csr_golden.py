"""Golden vectors for the sparse-key rank index, answered by the reference's own
CsrBase::rank / CsrBase::range (sparse_engine.hpp:79-97) through the harness
oracle/ref_csr.cpp (built by `make -f oracle/ref.mk oracle/_ref/csr_ref` from the
reference sources).  Run from the repository root:

    python tests/golden/make_csr_golden.py

Writes tests/golden/csr_golden.npz: per case the (class, amount) rows, the (i, j)
lookups and the reference's rank(i), rank(j), range(i, j)."""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
HARNESS = ROOT / "oracle" / "_ref" / "csr_ref"

# name: (class domain C, rows, lookups, seed, duplicates-heavy)
CASES = {
    "dense64k": (65536, 20000, 10000, 11, False),
    "small4k": (4096, 3000, 4000, 12, False),
    "ragged1000": (1000, 50, 2000, 13, True),
    "empty": (777, 0, 100, 14, False),
}


def make_case(C, nr, nq, seed, dup):
    rng = np.random.default_rng(seed)
    if dup:
        cls = rng.choice(rng.integers(0, C, 7), nr).astype(np.uint32)
    else:
        cls = (rng.zipf(1.2, nr) % C).astype(np.uint32) if nr else np.zeros(0, np.uint32)
    amt = rng.integers(-(1 << 40), 1 << 40, nr, dtype=np.int64)
    hi_lim = ((C + 63) // 64) * 64 + 70   # past the domain and the last bitmap word
    q = rng.integers(0, hi_lim, (nq, 2), dtype=np.int64)
    # exact support classes and their neighbours as endpoints
    if nr:
        k = nq // 4
        q[:k, 0] = cls[rng.integers(0, nr, k)]
        q[k:2 * k, 1] = cls[rng.integers(0, nr, k)].astype(np.int64) + 1
    return cls, amt, q


def run_reference(C, cls, amt, q):
    rows = np.zeros(len(cls), dtype=[("c", "<u4"), ("a", "<i8")])
    rows["c"], rows["a"] = cls, amt
    head = np.array([C], "<u4").tobytes() + np.array([len(cls), len(q)], "<u8").tobytes()
    out = subprocess.run([str(HARNESS)], input=head + rows.tobytes() + q.astype("<i8").tobytes(),
                         capture_output=True, check=True).stdout
    res = np.frombuffer(out, dtype=[("ra", "<i4"), ("rb", "<i4"), ("s", "<i8")])
    assert len(res) == len(q)
    return res


def main() -> int:
    if not HARNESS.exists():
        print(f"build the harness first: make -f oracle/ref.mk {HARNESS.relative_to(ROOT)}", file=sys.stderr)
        return 1
    arrays = {}
    for name, (C, nr, nq, seed, dup) in CASES.items():
        cls, amt, q = make_case(C, nr, nq, seed, dup)
        res = run_reference(C, cls, amt, q)
        arrays[f"{name}_C"] = np.array([C], np.int64)
        arrays[f"{name}_cls"] = cls
        arrays[f"{name}_amt"] = amt
        arrays[f"{name}_q"] = q
        arrays[f"{name}_rank_lo"] = res["ra"].astype(np.int64)
        arrays[f"{name}_rank_hi"] = res["rb"].astype(np.int64)
        arrays[f"{name}_range"] = res["s"].copy()
        print(name, C, nr, nq, int(res["s"].view(np.uint64).sum()))
    np.savez_compressed(ROOT / "tests" / "golden" / "csr_golden.npz", **arrays)
    return 0


if __name__ == "__main__":
    sys.exit(main())
