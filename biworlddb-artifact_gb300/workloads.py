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
* ``batched_trees`` (batched uneven trees): 4,096 independent version trees
  with lognormal state counts (median 2,000, sigma 1.6, capped at 200,000;
  about 30M states in all), each extending the previous state with p=0.95 or
  forking from a uniform earlier state, a key domain per tree drawn uniformly from
  the powers of two 1,024 ... 262,144, Poisson(8) events per state with Zipf s=1.1
  keys and delta = round(lognormal(7, 1)) with a negative sign at p=0.1, and
  1,000 range queries per tree (uniform states, uniform intervals).
* ``serving`` (request log of the served store): 2,000,000 requests on the
  trip-log tree -- 90% range-sum queries (version uniform among the versions that
  exist, lo uniform, width geometric with mean 1,024, clipped to the domain), 8%
  commits of 1-64 events (Zipf s=1.2 keys, delta = round(lognormal(7.3, 0.9))) to
  a uniformly chosen live leaf, 2% forks of a uniformly chosen existing version --
  with Poisson arrival times (unit rate; divide by the offered load).
* ``csr_lut`` (sparse-key rank index): 10,000,000 distinct u64 keys over
  [0, 2^40), 20,000,000 (key, delta) events on them, 100,000,000 point and
  100,000,000 range lookups, half present keys and half absent.
* ``csr_versioned`` (config 3's versioned dimension): the same keys, events and
  lookups on a 100,000-state chain with forks (extend with p=0.9, else fork from a
  uniform earlier state), events and lookups at uniform states.

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
REQUEST_DTYPE = np.dtype([("kind", "<u4"), ("version", "<u4"), ("lo", "<u4"), ("hi", "<u4"),
                          ("new_version", "<u4"), ("n_events", "<u4"), ("events_off", "<u8")])


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
    if name == "csr_versioned":
        return csr_versioned(seed=seed, scale=scale)
    if name == "batched_trees":
        return batched_trees(seed=seed, scale=scale)
    return CONFIGS[name](seed=seed, scale=scale)


@dataclass
class ForestWorkload:
    """Independent version trees concatenated: tree t owns states
    [state_off[t], state_off[t+1]) of ``parent`` (tree-local ids), events
    [event_off[t], event_off[t+1]) and queries [query_off[t], query_off[t+1]) (local
    states, keys in [0, n_keys[t]))."""
    name: str
    state_off: np.ndarray   # int64[T+1]
    event_off: np.ndarray   # int64[T+1]
    query_off: np.ndarray   # int64[T+1]
    n_keys: np.ndarray      # uint32[T]
    parent: np.ndarray      # int32[S]
    events: np.ndarray      # EVENT_DTYPE[E]
    queries: np.ndarray     # QUERY_DTYPE[Q]

    @property
    def n_trees(self) -> int:
        return int(self.n_keys.size)

    @property
    def algorithmic_bytes(self) -> int:
        """4S + 16E + 20Q: parent arrays, event records, query records + answers."""
        return 4 * len(self.parent) + 16 * len(self.events) + 20 * len(self.queries)

    def tree(self, t: int) -> Workload:
        s0, s1 = int(self.state_off[t]), int(self.state_off[t + 1])
        e0, e1 = int(self.event_off[t]), int(self.event_off[t + 1])
        q0, q1 = int(self.query_off[t]), int(self.query_off[t + 1])
        par = self.parent[s0:s1]
        chain = bool(np.all(par[1:] == np.arange(s1 - s0 - 1, dtype=np.int32)))
        return Workload(f"{self.name}[{t}]", par, int(self.n_keys[t]), self.events[e0:e1], self.queries[q0:q1],
                        chain)

    def describe(self) -> dict:
        sizes = np.diff(self.state_off)
        return {"workload": self.name, "trees": self.n_trees, "states": int(len(self.parent)),
                "events": int(len(self.events)), "queries": int(len(self.queries)),
                "states_per_tree": {"median": int(np.median(sizes)), "max": int(sizes.max()),
                                    "min": int(sizes.min())},
                "key_domains": sorted({int(c) for c in self.n_keys})}


_ZIPF_CACHE: dict = {}


def _zipf_table(C: int, s: float, seed: int):
    key = (C, s, seed)
    if key not in _ZIPF_CACHE:
        w = np.arange(1, C + 1, dtype=np.float64) ** (-s)
        cdf = np.cumsum(w)
        cdf /= cdf[-1]
        perm = np.random.default_rng((seed, C)).permutation(C).astype(np.uint32)
        _ZIPF_CACHE[key] = (cdf, perm)
    return _ZIPF_CACHE[key]


def batched_trees(seed: int = 0, scale: float = 1.0, *, trees: int = 4096, median: float = 2000.0,
                  sigma: float = 1.6, cap: int = 200_000, p_extend: float = 0.95, events_per_state: float = 8.0,
                  queries_per_tree: int = 1000, domain_bits=(10, 18), zipf: float = 1.1) -> ForestWorkload:
    """Batched uneven trees (``scale`` multiplies the tree count)."""
    rng = np.random.default_rng(seed)
    T = max(1, int(round(trees * scale)))
    sizes = np.clip(np.rint(rng.lognormal(np.log(median), sigma, size=T)), 2, cap).astype(np.int64)
    n_keys = (1 << rng.integers(domain_bits[0], domain_bits[1] + 1, size=T)).astype(np.uint32)
    state_off = np.zeros(T + 1, np.int64)
    np.cumsum(sizes, out=state_off[1:])
    S = int(state_off[-1])
    parent = np.empty(S, np.int32)
    counts = rng.poisson(events_per_state, size=S).astype(np.int64)
    for t in range(T):
        parent[state_off[t]:state_off[t + 1]] = _fork_tree(rng, int(sizes[t]), p_extend)
    cum = np.zeros(S + 1, np.int64)
    np.cumsum(counts, out=cum[1:])
    event_off = cum[state_off]
    E = int(event_off[-1])
    ev = np.empty(E, dtype=EVENT_DTYPE)
    Qt = int(queries_per_tree)
    qs = np.empty(T * Qt, dtype=QUERY_DTYPE)
    query_off = np.arange(T + 1, dtype=np.int64) * Qt
    for t in range(T):
        s0, s1 = int(state_off[t]), int(state_off[t + 1])
        e0, e1 = int(event_off[t]), int(event_off[t + 1])
        C = int(n_keys[t])
        n = e1 - e0
        ev["state"][e0:e1] = np.repeat(np.arange(s1 - s0, dtype=np.uint32), counts[s0:s1])
        cdf, perm = _zipf_table(C, zipf, seed)
        ranks = np.minimum(np.searchsorted(cdf, rng.random(n)), C - 1)
        ev["key"][e0:e1] = perm[ranks]
        d = np.rint(rng.lognormal(7.0, 1.0, size=n)).astype(np.int64)
        d[rng.random(n) < 0.1] *= -1
        ev["delta"][e0:e1] = d
        q = qs[t * Qt:(t + 1) * Qt]
        q["state"] = np.sort(rng.integers(0, s1 - s0, size=Qt)).astype(np.uint32)
        a = rng.integers(0, C + 1, size=Qt, dtype=np.int64)
        b = rng.integers(0, C + 1, size=Qt, dtype=np.int64)
        q["lo"], q["hi"] = np.minimum(a, b), np.maximum(a, b)
    return ForestWorkload("batched_trees", state_off, event_off, query_off, n_keys, parent, ev, qs)


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
    lookups, half present keys and half absent ones.  Index keys are the even values
    of the universe (2x a uniform draw over [0, 2^39)) and absent lookup keys odd
    ones, so membership is exact by construction with no search.  (The events'
    states do not enter the index, so none are drawn.)"""
    rng = np.random.default_rng(seed)
    K, E, L, bits = max(1, int(10_000_000 * scale)), max(1, int(20_000_000 * scale)), \
        max(2, int(100_000_000 * scale) if lookups is None else int(lookups)), 40
    half = 1 << (bits - 1)
    distinct = np.unique(rng.integers(0, half, size=int(K * 1.001) + 16, dtype=np.uint64))
    distinct = rng.permutation(distinct)[:K] * np.uint64(2)
    K = int(distinct.size)
    pick = np.concatenate([rng.permutation(K), rng.integers(0, K, size=max(0, E - K))])[:E]
    keys = distinct[pick]
    amounts = np.rint(rng.lognormal(7.3, 0.9, size=E)).astype(np.int64)
    amounts[rng.random(E) < 0.1] *= -1

    def mixed(n):
        out = rng.integers(0, half, size=n, dtype=np.uint64) * np.uint64(2) + np.uint64(1)   # absent: odd
        pres = rng.random(n) < 0.5
        out[pres] = distinct[rng.integers(0, K, size=int(pres.sum()))]
        return out

    point = mixed(L)
    a, b = mixed(L), mixed(L)
    ranges = np.stack([np.minimum(a, b), np.maximum(a, b)], axis=1)
    return CsrWorkload("csr_lut", bits, int(K), keys, amounts, point, ranges)


@dataclass
class CsrVersioned:
    """Config 3's versioned dimension: a version tree over sparse u64 keys.  Events
    (grouped by state) carry u64 keys; lookups are point and range lookups at states
    (grouped by state).  Answers are the usual root-path range sums over the keys."""
    name: str
    key_bits: int
    n_keys: int
    parent: np.ndarray
    ev_state: np.ndarray      # u32, non-decreasing
    ev_key: np.ndarray        # u64
    ev_delta: np.ndarray      # i64
    pt_state: np.ndarray      # u32, non-decreasing
    pt_key: np.ndarray        # u64
    rg_state: np.ndarray      # u32, non-decreasing
    rg_lo: np.ndarray         # u64
    rg_hi: np.ndarray         # u64


def csr_versioned(seed: int = 0, scale: float = 1.0, lookups: int | None = None) -> CsrVersioned:
    """The csr_lut keys, events and lookups (10M distinct u64 keys, 20M events, 100M
    point and 100M range lookups, half present and half absent) on a 100,000-state
    chain with forks (each state extends its parent with p=0.9, else forks from a
    uniform earlier state), events and lookups at uniform states."""
    base = csr_lut(seed, scale, lookups)
    rng = np.random.default_rng(seed + 1)
    S = max(2, int(100_000 * scale))
    parent = _fork_tree(rng, S, 0.9)
    E, L = len(base.keys), len(base.point)

    def states(n):
        return np.sort(rng.integers(0, S, size=n)).astype(np.uint32)
    return CsrVersioned("csr_versioned", base.key_bits, base.n_distinct, parent, states(E), base.keys,
                        base.amounts, states(L), base.point, states(L), base.ranges[:, 0].copy(),
                        base.ranges[:, 1].copy())


@dataclass
class ServeLog:
    """A request log on an initial tree: ``requests`` (REQUEST_DTYPE), the events of
    its commits (``commit_events``, EVENT_DTYPE, state = the created version) and
    unit-rate Poisson arrival times (``arrival``, seconds at 1 request/s)."""
    name: str
    base: Workload
    requests: np.ndarray
    commit_events: np.ndarray
    arrival: np.ndarray

    def describe(self) -> dict:
        k = self.requests["kind"]
        return {"workload": self.name, "initial_states": int(len(self.base.parent)),
                "initial_events": int(len(self.base.events)), "key_domain": int(self.base.n_keys),
                "requests": int(k.size), "queries": int((k == 0).sum()), "commits": int((k == 1).sum()),
                "forks": int((k == 2).sum()), "commit_events": int(len(self.commit_events))}

    def final_forest(self):
        """(parent, events grouped by state, queries grouped by state, order) of the
        tree after the whole log; order[i] is the request index of query row i."""
        base = self.base
        r = self.requests
        created = r["kind"] != 0
        S0 = len(base.parent)
        par = np.concatenate([base.parent, r["version"][created].astype(np.int32)])
        ev = np.concatenate([base.events, self.commit_events])
        qi = np.nonzero(r["kind"] == 0)[0]
        order = qi[np.argsort(r["version"][qi], kind="stable")]
        qs = np.empty(order.size, dtype=QUERY_DTYPE)
        qs["state"], qs["lo"], qs["hi"] = r["version"][order], r["lo"][order], r["hi"][order]
        assert np.all(np.diff(ev["state"].astype(np.int64)) >= 0) and par.size >= S0
        return par, ev, qs, order


def serving(seed: int = 0, scale: float = 1.0, *, requests: int = 2_000_000, base: Workload | None = None,
            p_query: float = 0.90, p_commit: float = 0.08, max_commit: int = 64,
            mean_width: float = 1024.0) -> ServeLog:
    """The serving request log on the trip-log tree (``scale`` shrinks the tree and
    the number of requests together)."""
    rng = np.random.default_rng(seed + 7)
    if base is None:
        base = trip_tree_base(seed, scale)
    C = base.n_keys
    n = max(1, int(round(requests * scale)))
    u = rng.random(n)
    kind = np.where(u < p_query, 0, np.where(u < p_query + p_commit, 1, 2)).astype(np.uint32)
    req = np.zeros(n, dtype=REQUEST_DTYPE)
    req["kind"] = kind
    S0 = len(base.parent)
    made = np.cumsum(kind != 0) - (kind != 0)          # versions created before request i
    avail = S0 + made
    q = kind == 0
    req["version"][q] = (rng.random(int(q.sum())) * avail[q]).astype(np.uint32)
    lo = rng.integers(0, C, size=int(q.sum()))
    width = rng.geometric(1.0 / mean_width, size=int(q.sum()))
    req["lo"][q], req["hi"][q] = lo, np.minimum(lo + width, C)
    # live leaves: versions without children; commits extend one, forks branch anywhere
    has_child = np.zeros(S0 + int((kind != 0).sum()), dtype=bool)
    has_child[base.parent[1:]] = True
    leaves = list(np.nonzero(~has_child[:S0])[0])
    pos = {int(v): i for i, v in enumerate(leaves)}
    nxt = S0
    ce_states, ce_n = [], []
    cw = np.cumsum(np.arange(1, C + 1, dtype=np.float64) ** -1.2)
    cw /= cw[-1]
    perm = rng.permutation(C).astype(np.uint32)
    for i in np.nonzero(kind != 0)[0]:
        if kind[i] == 1:
            j = int(rng.integers(0, len(leaves)))
            p = int(leaves[j])
            leaves[j] = nxt                                  # the leaf is extended
            pos.pop(p, None)
            pos[nxt] = j
            m = int(rng.integers(1, max_commit + 1))
            req["n_events"][i] = m
            req["events_off"][i] = sum(ce_n)
            ce_states.append(nxt)
            ce_n.append(m)
        else:
            p = int(rng.integers(0, nxt))
            if p in pos:                                     # a forked leaf stops being a leaf
                j = pos.pop(p)
                last = leaves.pop()
                if j < len(leaves):
                    leaves[j] = last
                    pos[int(last)] = j
            pos[nxt] = len(leaves)
            leaves.append(nxt)
        req["version"][i] = p
        req["new_version"][i] = nxt
        nxt += 1
    total = int(sum(ce_n))
    cev = np.empty(total, dtype=EVENT_DTYPE)
    cev["state"] = np.repeat(np.array(ce_states, dtype=np.uint32), ce_n) if total else []
    ranks = np.minimum(np.searchsorted(cw, rng.random(total)), C - 1)
    cev["key"] = perm[ranks]
    cev["delta"] = np.rint(rng.lognormal(7.3, 0.9, size=total)).astype(np.int64)
    arrival = np.cumsum(rng.exponential(1.0, size=n))
    return ServeLog("serving", base, req, cev, arrival)


def trip_tree_base(seed: int = 0, scale: float = 1.0) -> Workload:
    """The trip-log tree's states and events without its query batch."""
    rng = np.random.default_rng(seed)
    S, C = max(2, int(300_000 * scale)), 65536
    E = int(40_000_000 * scale)
    parent = _fork_tree(rng, S, 0.9)
    ev = np.empty(E, dtype=EVENT_DTYPE)
    ev["state"] = _grouped_states(rng, E, S)
    ev["key"] = _zipf_keys(rng, E, C, 1.2)
    ev["delta"] = np.rint(rng.lognormal(7.3, 0.9, size=E)).astype(np.int64)
    return Workload("trip_tree_base", parent, C, ev, np.empty(0, dtype=QUERY_DTYPE), False)
