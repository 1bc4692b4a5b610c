"""Seeded synthetic workloads for the event-model replay.

The reference measures its path on public datasets that are absent here; these
generators stand in with the shapes, sizes and value distributions of the
configured workloads:

* ``plain_chain`` (CPU-runnable plain replay): one linear chain of 20,000
  states, 1,000,000 events (state uniform over the chain, key Zipf s=1.1 over a
  4,096-key domain, delta = round(lognormal(7, 1)) with a negative sign at
  p=0.1), 10,000 queries (state uniform, lo uniform, width geometric with mean
  256, clipped to the domain).
* ``trip_tree`` (trip-log-shaped single tree): 300,000 states where each new
  state extends the previous one with p=0.9 or forks from a uniformly chosen
  earlier state, 40,000,000 events with Zipf s=1.2 keys over 65,536 cells and
  delta = round(lognormal(7.3, 0.9)), 50,000,000 queries at uniform states with
  uniform intervals.

Events and queries are produced grouped by state (a commit log appends each
version's events when the version is created; answers come back state-major, as
the reference's answer vectors are ordered).  Keys of the Zipf distributions are
scattered over the domain by a fixed seeded permutation, so hot cells are not
adjacent.  Everything is a pure function of (config, seed, scale).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

EVENT_DTYPE = np.dtype([("state", "<u4"), ("key", "<u4"), ("delta", "<i8")])
QUERY_DTYPE = np.dtype([("state", "<u4"), ("lo", "<u4"), ("hi", "<u4")])


@dataclass
class Workload:
    name: str
    parent: np.ndarray      # int32[S]
    n_keys: int
    events: np.ndarray      # EVENT_DTYPE[E], grouped by state
    queries: np.ndarray     # QUERY_DTYPE[Q], grouped by state
    chain: bool

    @property
    def algorithmic_bytes(self) -> int:
        """4S + 16E + 20Q: parent array, event records, query records + answers."""
        return 4 * len(self.parent) + 16 * len(self.events) + 20 * len(self.queries)

    def describe(self) -> dict:
        return {"workload": self.name, "states": int(len(self.parent)), "events": int(len(self.events)),
                "queries": int(len(self.queries)), "key_domain": int(self.n_keys),
                "topology": "chain" if self.chain else "tree"}


def _zipf_keys(rng, n, C, s):
    w = np.arange(1, C + 1, dtype=np.float64) ** (-s)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    ranks = np.searchsorted(cdf, rng.random(n))
    np.minimum(ranks, C - 1, out=ranks)
    perm = rng.permutation(C).astype(np.uint32)
    return perm[ranks]


def _fork_tree(rng, S, p_extend):
    v = np.arange(S, dtype=np.int64)
    parent = v - 1
    fork = rng.random(S) >= p_extend
    fork[:2] = False
    idx = np.nonzero(fork)[0]
    parent[idx] = (rng.random(idx.size) * idx).astype(np.int64)
    parent[0] = -1
    return parent.astype(np.int32)


def _grouped_states(rng, n, S):
    counts = np.bincount(rng.integers(0, S, size=n), minlength=S)
    return np.repeat(np.arange(S, dtype=np.uint32), counts)


def plain_chain(seed: int = 0, scale: float = 1.0) -> Workload:
    rng = np.random.default_rng(seed)
    S, C = max(2, int(20_000 * scale)), 4096
    E, Q = int(1_000_000 * scale), max(1, int(10_000 * scale))
    parent = (np.arange(S, dtype=np.int64) - 1).astype(np.int32)
    ev = np.empty(E, dtype=EVENT_DTYPE)
    ev["state"] = _grouped_states(rng, E, S)
    ev["key"] = _zipf_keys(rng, E, C, 1.1)
    d = np.rint(rng.lognormal(7.0, 1.0, size=E)).astype(np.int64)
    d[rng.random(E) < 0.1] *= -1
    ev["delta"] = d
    qs = np.empty(Q, dtype=QUERY_DTYPE)
    qs["state"] = _grouped_states(rng, Q, S)
    lo = rng.integers(0, C, size=Q)
    width = rng.geometric(1.0 / 256.0, size=Q)
    qs["lo"], qs["hi"] = lo, np.minimum(lo + width, C)
    return Workload("plain_chain", parent, C, ev, qs, True)


def trip_tree(seed: int = 0, scale: float = 1.0) -> Workload:
    rng = np.random.default_rng(seed)
    S, C = max(2, int(300_000 * scale)), 65536
    E, Q = int(40_000_000 * scale), int(50_000_000 * scale)
    parent = _fork_tree(rng, S, 0.9)
    ev = np.empty(E, dtype=EVENT_DTYPE)
    ev["state"] = _grouped_states(rng, E, S)
    ev["key"] = _zipf_keys(rng, E, C, 1.2)
    ev["delta"] = np.rint(rng.lognormal(7.3, 0.9, size=E)).astype(np.int64)
    qs = np.empty(Q, dtype=QUERY_DTYPE)
    qs["state"] = _grouped_states(rng, Q, S)
    a = rng.integers(0, C + 1, size=Q, dtype=np.int64)
    b = rng.integers(0, C + 1, size=Q, dtype=np.int64)
    qs["lo"], qs["hi"] = np.minimum(a, b), np.maximum(a, b)
    return Workload("trip_tree", parent, C, ev, qs, False)


CONFIGS = {"plain_chain": plain_chain, "trip_tree": trip_tree}


def make(name: str, seed: int = 0, scale: float = 1.0) -> Workload:
    return CONFIGS[name](seed=seed, scale=scale)
