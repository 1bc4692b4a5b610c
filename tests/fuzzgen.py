"""Randomized branching fuzz cases -- TEST INFRASTRUCTURE.

A restatement of the reference fuzz harness's case generator
(fuzz_fullpath.cpp:46-64 SplitMix64 ``FRng``, :162-320 ``build_case``, :362-387 the
per-case parameter draw): a fresh tiny BWBASE02 fixture and an explicit declared
workload per case.  Profiles (fuzz_fullpath.cpp:373-383): 0 row-heavy, 1
factor-heavy, 2 forced empty ranges, 3 inserts/moves at t_max+1, 4 negative
amounts, 5 factor edits to 0, 6 negative factors, 7 all factor edits, 8 a dense
8-tick frame, 9 mixed.  The first 60 cases are the deterministic edge cases (10
profiles x 3 topologies x 2 range scopes); the rest draw their profile, topology,
q and scope at random.  Parents follow common.hpp:219-226 (chain, bushy, star).

``case(ci, states)`` returns a ``FuzzCase`` whose fixture image and answers are
pinned by tests/golden/fuzz_golden.json (made by the reference's own build_case
and "rf" arm, oracle/ref_fuzz.cpp).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

M64 = (1 << 64) - 1
GOLDEN = 0x9E3779B97F4A7C15
OP_REPLACE, OP_INSERT, OP_DELETE, OP_MOVE, OP_FACTOR = 0, 1, 2, 3, 4
PROFILES = ["row-heavy", "factor-heavy", "empty-ranges", "tmax1-inserts", "neg-amounts", "zero-factor",
            "neg-factor", "all-factor", "dense-frame", "mixed"]
HDR = struct.Struct("<8s q i i q q q q q")


class FRng:
    """SplitMix64 with the fuzz harness's helpers (fuzz_fullpath.cpp:46-64)."""

    def __init__(self, seed: int):
        seed &= M64
        self.s = seed if seed else GOLDEN

    def next(self) -> int:
        self.s = (self.s + GOLDEN) & M64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
        return z ^ (z >> 31)

    def range(self, lo: int, hi: int) -> int:   # half-open [lo, hi)
        if hi <= lo:
            return lo
        return lo + self.next() % (hi - lo)

    def bounded(self, n: int) -> int:
        return self.next() % n if n > 0 else 0

    def chance(self, pct: int) -> bool:
        return self.next() % 100 < pct


def version_parent(topology: int, v: int) -> int:
    if v <= 0:
        return -1
    return v - 1 if topology == 0 else (v - 1) // 2 if topology == 1 else 0


@dataclass
class FuzzCase:
    index: int
    seed: int
    profile: int
    topology: int
    q: int
    per_state: bool
    N: int
    G: int
    p_factor: int
    states: int
    fixture: bytes = b""
    parent: np.ndarray = field(default=None)
    op: np.ndarray = field(default=None)
    g: np.ndarray = field(default=None)
    id: np.ndarray = field(default=None)
    val: np.ndarray = field(default=None)
    t: np.ndarray = field(default=None)
    qlo: np.ndarray = field(default=None)
    qhi: np.ndarray = field(default=None)
    ins_t: np.ndarray = field(default=None)
    ins_g: np.ndarray = field(default=None)

    @property
    def name(self) -> str:
        return (f"c{self.index}-{PROFILES[self.profile]}-t{self.topology}-q{self.q}-"
                f"{'ps' if self.per_state else 'shared'}")


def case(ci: int, states: int = 33) -> FuzzCase:
    seed = (ci * 0x2545F4914F6CDD1D + 12345) & M64
    r = FRng(seed ^ 0xABCDEF)
    if ci < 60:
        prof, topo, per_state, q = ci % 10, (ci // 10) % 3, (ci // 30) % 2 == 0, 1 + (ci // 6) % 3
    else:
        prof = r.bounded(10)
        topo = r.bounded(3)
        q = 1 + r.bounded(3)
        per_state = r.chance(55)
    N = 12 + r.bounded(40)
    G = 2 + r.bounded(3)
    span, dense, tmax1, empty, neg_amt, zero_f, neg_f, p_factor = 1000000, False, False, False, False, False, False, 25
    if prof == 0:
        p_factor = 10 + r.bounded(20)
    elif prof == 1:
        p_factor = 50 + r.bounded(30)
    elif prof == 2:
        empty = True
    elif prof == 3:
        tmax1, p_factor = True, 20
    elif prof == 4:
        neg_amt, p_factor = True, 20
    elif prof == 5:
        zero_f, p_factor = True, 60
    elif prof == 6:
        neg_f, p_factor = True, 60
    elif prof == 7:
        p_factor = 100
    elif prof == 8:
        span, dense, p_factor = 8, True, 30
    c = FuzzCase(ci, seed, prof, topo, q, per_state, N, G, p_factor, states)

    # ---- fixture (build_case, fuzz_fullpath.cpp:165-186)
    rng = FRng(seed ^ 0x5DEECE66D)
    tmin0 = 1000000
    span = 8 if dense else span
    fac = [1000 if dense else 1 + rng.bounded(2000) for _ in range(G)]
    rows = []
    for _ in range(N):
        t = tmin0 + (rng.range(0, span + 1) if span > 0 else 0)
        amt = rng.range(-1000000, 1000000)
        if not neg_amt:
            amt = abs(amt) + 1
        rows.append((t, amt, rng.bounded(G)))
    t_min = min(x[0] for x in rows)
    t_max = max(x[0] for x in rows)
    img = bytearray(HDR.pack(b"BWBASE02", N, G, 0, N, 0, t_min, t_max, 6))
    for t, amt, g in rows:
        img += struct.pack("<qqii", t, amt, g, 0)
    img += struct.pack(f"<{G}q", *fac) + struct.pack(f"<{G}i", *range(G))
    c.fixture = bytes(img)
    hi_max = t_max + 1

    # ---- parents and edits (fuzz_fullpath.cpp:196-259)
    S = states
    c.parent = np.array([version_parent(topo, v) for v in range(S)], dtype=np.int32)
    op = np.zeros(S, np.uint8)
    eg = np.zeros(S, np.int32)
    eid = np.zeros(S, np.int64)
    ev = np.zeros(S, np.int64)
    et = np.zeros(S, np.int64)
    ins_t, ins_g = [], []

    def amount() -> int:
        v = rng.range(-2000000, 2000000)
        return v if neg_amt else abs(v)

    for v in range(1, S):
        if rng.chance(p_factor):
            op[v] = OP_FACTOR
            eg[v] = rng.bounded(G)
            if zero_f and rng.chance(60):
                val = 0
            elif neg_f and rng.chance(60):
                val = -(1 + rng.bounded(5000))
            elif rng.chance(40):
                val = 0
            elif rng.chance(50):
                val = -(1 + rng.bounded(2000))
            else:
                val = 1 + rng.bounded(5000)
            ev[v] = val
            continue
        roll = rng.bounded(100)
        if roll < 50:
            op[v], eid[v] = OP_REPLACE, rng.range(0, N)
            ev[v] = amount()
        elif roll < 70:
            op[v], eid[v] = OP_INSERT, N + len(ins_t)
            et[v] = t_max + 1 if (tmax1 and rng.chance(70)) else rng.range(t_min, hi_max)
            eg[v] = rng.bounded(G)
            ev[v] = amount()
            ins_t.append(int(et[v]))
            ins_g.append(int(eg[v]))
        elif roll < 85:
            op[v], eid[v] = OP_DELETE, rng.range(0, N)
        else:
            op[v], eid[v] = OP_MOVE, rng.range(0, N)
            et[v] = t_max + 1 if (tmax1 and rng.chance(50)) else rng.range(t_min, hi_max)
            eg[v] = rng.bounded(G)
            ev[v] = amount()
    c.op, c.g, c.id, c.val, c.t = op, eg, eid, ev, et
    c.ins_t = np.array(ins_t, dtype=np.int64)
    c.ins_g = np.array(ins_g, dtype=np.int32)

    # ---- declared ranges (fuzz_fullpath.cpp:262-283)
    def gen_range(qr: FRng):
        if empty and qr.chance(70):
            x = qr.range(t_min, hi_max + 1)
            return x, x
        lo = qr.range(t_min, hi_max)
        hi = qr.range(lo, hi_max + 1)
        return lo, max(hi, lo)

    if per_state:
        qlo = np.zeros(S * q, np.int64)
        qhi = np.zeros(S * q, np.int64)
        for v in range(1, S):
            qr = FRng(seed ^ ((v * GOLDEN) & M64) ^ 0xC0FFEE)
            for k in range(q):
                qlo[v * q + k], qhi[v * q + k] = gen_range(qr)
    else:
        qr = FRng(seed ^ 0xBEEF)
        pairs = [gen_range(qr) for _ in range(q)]
        qlo = np.array([p[0] for p in pairs], np.int64)
        qhi = np.array([p[1] for p in pairs], np.int64)
    c.qlo, c.qhi = qlo, qhi
    return c
