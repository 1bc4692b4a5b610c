"""Random event-model cases for the parity tests (numpy, seeded).

Trees: chain (parent v-1), bushy (binary heap (v-1)//2), star (root), and
"forking" trees where each new state extends the previous one with probability
p_extend or forks from a uniformly chosen earlier state (common.hpp:219-226 for
the first three; the trip-log tree shape for the last).
"""
from __future__ import annotations

import numpy as np

EVENT_DTYPE = np.dtype([("state", "<u4"), ("key", "<u4"), ("delta", "<i8")])
QUERY_DTYPE = np.dtype([("state", "<u4"), ("lo", "<u4"), ("hi", "<u4")])


def make_tree(S: int, kind: str, rng: np.random.Generator, p_extend: float = 0.9) -> np.ndarray:
    v = np.arange(S, dtype=np.int64)
    if kind == "chain":
        p = v - 1
    elif kind == "bushy":
        p = (v - 1) // 2
    elif kind == "star":
        p = np.zeros(S, dtype=np.int64)
    elif kind == "fork":
        p = v - 1
        fork = rng.random(S) >= p_extend
        fork[:2] = False
        idx = np.nonzero(fork)[0]
        p[idx] = (rng.random(idx.size) * idx).astype(np.int64)
    else:
        raise ValueError(kind)
    p[0] = -1
    return p.astype(np.int32)


def make_events(S: int, C: int, E: int, rng, zipf: float = 0.0, neg_frac: float = 0.1,
                big: bool = False) -> np.ndarray:
    ev = np.empty(E, dtype=EVENT_DTYPE)
    ev["state"] = np.sort(rng.integers(0, S, size=E)).astype(np.uint32)
    if zipf > 0:
        w = 1.0 / np.arange(1, C + 1) ** zipf
        cdf = np.cumsum(w)
        cdf /= cdf[-1]
        ranks = np.minimum(np.searchsorted(cdf, rng.random(E)), C - 1)
        perm = rng.permutation(C)
        ev["key"] = perm[ranks].astype(np.uint32)
    else:
        ev["key"] = rng.integers(0, C, size=E).astype(np.uint32)
    if big:  # full-range int64 deltas: exercises two's-complement wrap
        d = rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, size=E, dtype=np.int64)
    else:
        d = np.rint(rng.lognormal(7.0, 1.0, size=E)).astype(np.int64)
        d[rng.random(E) < neg_frac] *= -1
    ev["delta"] = d
    return ev


def make_queries(S: int, C: int, Q: int, rng, empty_frac: float = 0.05,
                 full_frac: float = 0.05) -> np.ndarray:
    qs = np.empty(Q, dtype=QUERY_DTYPE)
    qs["state"] = np.sort(rng.integers(0, S, size=Q)).astype(np.uint32)
    a = rng.integers(0, C + 1, size=Q)
    b = rng.integers(0, C + 1, size=Q)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    r = rng.random(Q)
    emp = r < empty_frac          # empty and reversed intervals answer 0
    hi[emp] = lo[emp] - (lo[emp] > 0)
    full = (r >= empty_frac) & (r < empty_frac + full_frac)
    lo[full], hi[full] = 0, C
    qs["lo"], qs["hi"] = lo.astype(np.uint32), hi.astype(np.uint32)
    return qs


def to_device(torch, parent, events, queries, device="cuda"):
    p = torch.from_numpy(np.ascontiguousarray(parent, dtype=np.int32)).to(device)
    e = torch.from_numpy(np.ascontiguousarray(events).view(np.int64).reshape(-1, 2)).to(device)
    q = torch.from_numpy(np.ascontiguousarray(queries).view(np.int32).reshape(-1, 3)).to(device)
    return p, e, q
