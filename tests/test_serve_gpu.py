"""GPU parity of the served version store (bw_serve_* through the C ABI): request
logs of queries, commits and forks served by the persistent loop against the
oracle's replay of the final tree; the same answers alone and in the mix; tight
memory caps (sparse checkpoints, long overlay lists), overlay lists longer than a
warp (linked lists), admission refusals and malformed logs."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_base(bw, seed, S=3000, E=300_000):
    rng = np.random.default_rng(seed)
    w = bw.workloads
    parent = w._fork_tree(rng, S, 0.9)
    ev = np.empty(E, dtype=w.EVENT_DTYPE)
    ev["state"] = w._grouped_states(rng, E, S)
    ev["key"] = w._zipf_keys(rng, E, 65536, 1.2)
    ev["delta"] = np.rint(rng.lognormal(7.3, 0.9, size=E)).astype(np.int64)
    return w.Workload("base", parent, 65536, ev, np.empty(0, dtype=w.QUERY_DTYPE), False)


def oracle_answers(oracle_mod, log):
    par, ev, qs, order = log.final_forest()
    got = oracle_mod.ev_sweep(par, log.base.n_keys, ev, qs)
    out = np.zeros(len(log.requests), dtype=np.int64)
    out[order] = got
    return out


def server_for(bw, log, cap=8 << 30, chain=0, extra_versions=0, extra_events=0):
    b = log.base
    return bw.Server(b.parent, b.n_keys, b.events, max_versions=len(b.parent) + len(log.requests) + extra_versions,
                     max_events=len(b.events) + len(log.commit_events) + extra_events, hbm_cap_bytes=cap,
                     chain_limit=chain)


@pytest.mark.parametrize("rate,inflight", [(None, 1 << 16), (2e6, 1 << 16), (5e5, 64)])
def test_serve_matches_oracle(bw, torch_cuda, oracle_mod, rate, inflight):
    log = bw.workloads.serving(3, base=small_base(bw, 3), requests=30_000)
    want = oracle_answers(oracle_mod, log)
    srv = server_for(bw, log)
    arr = None if rate is None else log.arrival / rate
    ans, lat, st = srv.run(log.requests, log.commit_events, arr, max_inflight=inflight)
    q = log.requests["kind"] == 0
    np.testing.assert_array_equal(ans[q], want[q])
    assert np.all(lat > 0) and st["requests"] == len(log.requests) and st["queries"] == int(q.sum())
    srv.close()


def test_alone_equals_mix(bw, torch_cuda, oracle_mod):
    """Each answer is the same when its request runs alone as when it runs in the mix."""
    log = bw.workloads.serving(4, base=small_base(bw, 4), requests=20_000)
    srv = server_for(bw, log)
    mixed, _, _ = srv.run(log.requests, log.commit_events, log.arrival / 3e6)
    srv.reset()
    create = np.nonzero(log.requests["kind"] != 0)[0]
    srv.run(log.requests[create], log.commit_events)            # the same versions, no queries
    rng = np.random.default_rng(0)
    qi = rng.choice(np.nonzero(log.requests["kind"] == 0)[0], size=60, replace=False)
    for i in qi:
        alone, _, _ = srv.run(log.requests[i:i + 1])
        assert alone[0] == mixed[i]
    want = oracle_answers(oracle_mod, log)
    np.testing.assert_array_equal(mixed[qi], want[qi])
    srv.close()


def test_tight_cap_sparse_checkpoints(bw, torch_cuda, oracle_mod):
    log = bw.workloads.serving(5, base=small_base(bw, 5, S=4000, E=200_000), requests=20_000)
    row = (65536 + 1) * 8
    srv = server_for(bw, log, cap=200 * row + (64 << 20))
    info = srv.info()
    assert info["spacing"] >= 8 and info["store_bytes"] <= 200 * row + (64 << 20)
    ans, _, _ = srv.run(log.requests, log.commit_events)
    q = log.requests["kind"] == 0
    np.testing.assert_array_equal(ans[q], oracle_answers(oracle_mod, log)[q])
    srv.close()


def test_long_commit_chains_link_lists(bw, torch_cuda, oracle_mod):
    """More than 32 successive commits on one leaf: overlay lists continue by link."""
    w = bw.workloads
    base = small_base(bw, 6, S=500, E=20_000)
    rng = np.random.default_rng(6)
    S0, n_commit = len(base.parent), 150
    leaf = S0 - 1 if base.parent[S0 - 1] != S0 - 2 or True else 0
    reqs, cev, off = [], [], 0
    v = leaf
    for k in range(n_commit):
        m = int(rng.integers(1, 65))
        reqs.append((1, v, 0, 0, S0 + k, m, off))
        e = np.empty(m, dtype=w.EVENT_DTYPE)
        e["state"], e["key"] = S0 + k, rng.integers(0, 65536, m)
        e["delta"] = rng.integers(-10**6, 10**6, m)
        cev.append(e)
        off += m
        v = S0 + k
        for _ in range(3):
            lo = int(rng.integers(0, 65536))
            reqs.append((0, int(rng.integers(0, S0 + k + 1)), lo, min(65536, lo + int(rng.integers(1, 40000))), 0, 0, 0))
    req = np.array(reqs, dtype=w.REQUEST_DTYPE)
    log = w.ServeLog("chain", base, req, np.concatenate(cev), np.arange(len(req), dtype=np.float64))
    srv = server_for(bw, log)
    ans, _, _ = srv.run(log.requests, log.commit_events)
    q = req["kind"] == 0
    np.testing.assert_array_equal(ans[q], oracle_answers(oracle_mod, log)[q])
    srv.close()


def test_admission_and_malformed_logs(bw, torch_cuda):
    log = bw.workloads.serving(7, base=small_base(bw, 7, S=800, E=40_000), requests=5_000)
    b = log.base
    srv = bw.Server(b.parent, b.n_keys, b.events, max_versions=len(b.parent) + len(log.requests),
                    max_events=len(b.events) + 10, hbm_cap_bytes=8 << 30)
    with pytest.raises(RuntimeError):   # commit events beyond the free arena: refused
        srv.run(log.requests, log.commit_events)
    bad = log.requests[:1].copy()
    bad["kind"], bad["version"] = 0, len(b.parent) + 5     # a version that does not exist yet
    with pytest.raises(RuntimeError):
        srv.run(bad)
    srv.close()
    with pytest.raises(RuntimeError):   # the store itself over the cap
        bw.Server(b.parent, b.n_keys, b.events, max_versions=len(b.parent), max_events=len(b.events),
                  hbm_cap_bytes=1 << 20)


def _late_arrivals(log, cut):
    """Arrival times that publish only the first `cut` requests within the run."""
    arr = np.zeros(len(log.requests))
    arr[cut:] = 1e4
    return arr


def test_serve_host_timeout_stops_loop(bw, torch_cuda, oracle_mod):
    """A host timeout while requests are still unpublished: the host raises the abort
    word, the loop's bounded waits see it and return, the run reports an error, and
    the store and context stay usable."""
    import time
    log = bw.workloads.serving(6, base=small_base(bw, 6), requests=4_000)
    srv = server_for(bw, log)
    t0 = time.perf_counter()
    with pytest.raises(RuntimeError, match="1001"):
        srv.run(log.requests, log.commit_events, _late_arrivals(log, 1500), timeout_s=0.5)
    assert time.perf_counter() - t0 < 20.0
    srv.reset()
    ans, _, _ = srv.run(log.requests, log.commit_events)
    q = log.requests["kind"] == 0
    np.testing.assert_array_equal(ans[q], oracle_answers(oracle_mod, log)[q])
    srv.close()


def test_serve_device_wait_limit_stops_loop(bw, torch_cuda, oracle_mod):
    """A device wait that reaches its poll limit (requests that never arrive within
    it): the loop records the error word and returns before the host timeout; a new
    store on the same context then serves the full log exactly."""
    import time
    log = bw.workloads.serving(7, base=small_base(bw, 7), requests=4_000)
    b = log.base
    srv = bw.Server(b.parent, b.n_keys, b.events, max_versions=len(b.parent) + len(log.requests),
                    max_events=len(b.events) + len(log.commit_events), hbm_cap_bytes=8 << 30, spin_limit=4000)
    t0 = time.perf_counter()
    with pytest.raises(RuntimeError, match="1001"):
        srv.run(log.requests, log.commit_events, _late_arrivals(log, 1000), timeout_s=60.0)
    assert time.perf_counter() - t0 < 30.0
    srv.close()
    srv = server_for(bw, log)
    ans, _, _ = srv.run(log.requests, log.commit_events)
    q = log.requests["kind"] == 0
    np.testing.assert_array_equal(ans[q], oracle_answers(oracle_mod, log)[q])
    srv.close()
