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
* ``csr_lut`` (sparse-key rank index): 10,000,000 distinct u64 keys over
  [0, 2^40), 20,000,000 (key, delta) events on them, 100,000,000 point and
  100,000,000 range lookups, half present keys and half absent.

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


def make(name: str, seed: int = 0, scale: float = 1.0):
    if name == "csr_lut":
        return csr_lut(seed=seed, scale=scale)
    return CONFIGS[name](seed=seed, scale=scale)


@dataclass
class CsrWorkload:
    """Sparse-key rank-index workload: `keys`/`amounts` are the event (key, delta)
    pairs the index is built from; `point` lookups and `ranges` [lo, hi) pairs are
    each half present keys and half absent ones."""
    name: str
    key_bits: int
    n_distinct: int
    keys: np.ndarray        # u64[E]
    amounts: np.ndarray     # int64[E]
    point: np.ndarray       # u64[L]
    ranges: np.ndarray      # u64[L, 2], lo <= hi

    def describe(self) -> dict:
        return {"workload": self.name, "distinct_keys": self.n_distinct, "events": int(len(self.keys)),
                "point_lookups": int(len(self.point)), "range_lookups": int(len(self.ranges)),
                "key_universe_bits": self.key_bits}


def csr_lut(seed: int = 0, scale: float = 1.0, lookups: int | None = None) -> CsrWorkload:
    """10,000,000 distinct u64 keys uniform over [0, 2^40), 20,000,000 events on them
    (every key at least once, the rest uniform; delta = round(lognormal(7.3, 0.9))
    with a negative sign at p=0.1), 100,000,000 point lookups and 100,000,000 range
    lookups, half present keys and half absent ones.  (The events' states do not
    enter the index, so none are drawn.)"""
    rng = np.random.default_rng(seed)
    K, E, L, bits = max(1, int(10_000_000 * scale)), max(1, int(20_000_000 * scale)), \
        max(2, int(100_000_000 * scale) if lookups is None else int(lookups)), 40
    universe = 1 << bits
    distinct = np.unique(rng.integers(0, universe, size=int(K * 1.001) + 16, dtype=np.uint64))
    distinct = rng.permutation(distinct)[:K]
    pick = np.concatenate([rng.permutation(K), rng.integers(0, K, size=max(0, E - K))])[:E]
    keys = distinct[pick]
    amounts = np.rint(rng.lognormal(7.3, 0.9, size=E)).astype(np.int64)
    amounts[rng.random(E) < 0.1] *= -1

    present_sorted = np.sort(distinct)

    def absent(n):
        x = rng.integers(0, universe, size=n, dtype=np.uint64)
        hit = present_sorted[np.minimum(np.searchsorted(present_sorted, x), K - 1)] == x
        while hit.any():
            x[hit] = rng.integers(0, universe, size=int(hit.sum()), dtype=np.uint64)
            hit = present_sorted[np.minimum(np.searchsorted(present_sorted, x), K - 1)] == x
        return x

    def mixed(n):
        out = np.empty(n, np.uint64)
        pres = rng.random(n) < 0.5
        out[pres] = distinct[rng.integers(0, K, size=int(pres.sum()))]
        out[~pres] = absent(int((~pres).sum()))
        return out

    point = mixed(L)
    a, b = mixed(L), mixed(L)
    ranges = np.stack([np.minimum(a, b), np.maximum(a, b)], axis=1)
    return CsrWorkload("csr_lut", bits, int(K), keys, amounts, point, ranges)
