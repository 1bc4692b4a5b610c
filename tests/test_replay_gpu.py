"""GPU parity of the event-model replay (libbwgpu.so through the C ABI) against
the oracle on seeded inputs: chains, bushy/star/forking trees, hot Zipf keys,
wrapping int64 deltas, multi-slice and multi-window key domains, degenerate
shapes, and inputs the device must reject without faulting."""
from __future__ import annotations

import numpy as np
import pytest

import evgen

pytestmark = pytest.mark.gpu


def run(bw, torch, parent, C, ev, qs, **kw):
    p, e, q = evgen.to_device(torch, parent, ev, qs)
    return bw.replay(p, C, e, q, **kw).cpu().numpy()


CASES = [
    # kind, S, C, E, Q, zipf, blocks
    ("chain", 500, 64, 6000, 4000, 0.0, 0),
    ("chain", 3000, 4096, 60000, 40000, 1.1, 0),
    ("chain", 3000, 4096, 60000, 40000, 1.1, 7),
    ("bushy", 2049, 1000, 30000, 20000, 0.0, 0),
    ("star", 2049, 1000, 30000, 20000, 0.0, 5),
    ("fork", 5000, 65536, 120000, 90000, 1.2, 0),
    ("fork", 5000, 65536, 120000, 90000, 1.2, 1),
    ("fork", 20000, 3000, 200000, 150000, 1.2, 0),
]


@pytest.mark.parametrize("kind,S,C,E,Q,zipf,blocks", CASES)
def test_replay_matches_oracle(bw, torch_cuda, oracle_mod, kind, S, C, E, Q, zipf, blocks):
    rng = np.random.default_rng(S + C + E)
    parent = evgen.make_tree(S, kind, rng)
    ev = evgen.make_events(S, C, E, rng, zipf=zipf)
    qs = evgen.make_queries(S, C, Q, rng)
    want = oracle_mod.ev_sweep(parent, C, ev, qs)
    got = run(bw, torch_cuda, parent, C, ev, qs, blocks=blocks)
    np.testing.assert_array_equal(got, want)


def test_chain_hint_matches_tree_path(bw, torch_cuda, oracle_mod):
    rng = np.random.default_rng(7)
    S, C = 4000, 20000
    parent = evgen.make_tree(S, "chain", rng)
    ev = evgen.make_events(S, C, 80000, rng, zipf=1.1)
    qs = evgen.make_queries(S, C, 50000, rng)
    want = oracle_mod.ev_blocks(parent, C, ev, qs, blocks=8)
    np.testing.assert_array_equal(run(bw, torch_cuda, parent, C, ev, qs, chain=True), want)
    np.testing.assert_array_equal(run(bw, torch_cuda, parent, C, ev, qs, chain=False), want)


def test_wrapping_int64(bw, torch_cuda, oracle_mod):
    rng = np.random.default_rng(9)
    S, C = 1500, 777
    parent = evgen.make_tree(S, "fork", rng)
    ev = evgen.make_events(S, C, 30000, rng, big=True)
    qs = evgen.make_queries(S, C, 20000, rng)
    np.testing.assert_array_equal(run(bw, torch_cuda, parent, C, ev, qs),
                                  oracle_mod.ev_bruteforce(parent, ev, qs))


def test_hot_key(bw, torch_cuda, oracle_mod):
    # every event on one key: maximal contention in the warp-aggregated updates
    rng = np.random.default_rng(2)
    S, C = 3000, 1000
    parent = evgen.make_tree(S, "fork", rng)
    ev = evgen.make_events(S, C, 60000, rng)
    ev["key"] = 517
    qs = evgen.make_queries(S, C, 30000, rng)
    np.testing.assert_array_equal(run(bw, torch_cuda, parent, C, ev, qs, blocks=3),
                                  oracle_mod.ev_sweep(parent, C, ev, qs))


def test_multi_slice_block(bw, torch_cuda, oracle_mod):
    # one block with far more distinct keys than fit one shared-memory slice
    rng = np.random.default_rng(4)
    S, C = 800, 1 << 17
    parent = evgen.make_tree(S, "chain", rng)
    ev = evgen.make_events(S, C, 150000, rng)
    qs = evgen.make_queries(S, C, 40000, rng)
    np.testing.assert_array_equal(run(bw, torch_cuda, parent, C, ev, qs, blocks=1),
                                  oracle_mod.ev_sweep(parent, C, ev, qs))


def test_multi_window_domain(bw, torch_cuda, oracle_mod):
    # key domain wider than one 2^18-key bitmap window, ragged last word
    rng = np.random.default_rng(6)
    S, C = 1200, (1 << 19) + 13
    parent = evgen.make_tree(S, "fork", rng)
    ev = evgen.make_events(S, C, 50000, rng)
    ev["key"][:50] = C - 1
    qs = evgen.make_queries(S, C, 30000, rng)
    np.testing.assert_array_equal(run(bw, torch_cuda, parent, C, ev, qs, blocks=2),
                                  oracle_mod.ev_sweep(parent, C, ev, qs))


def test_big_root_step(bw, torch_cuda, oracle_mod):
    # the base relation: one state with far more events than a CTA has threads
    rng = np.random.default_rng(8)
    S, C = 300, 5000
    parent = evgen.make_tree(S, "bushy", rng)
    ev = evgen.make_events(S, C, 20000, rng)
    ev["state"][:15000] = 0
    ev.sort(order="state", kind="stable")
    qs = evgen.make_queries(S, C, 5000, rng)
    qs["state"][:2000] = 7
    qs.sort(order="state", kind="stable")
    np.testing.assert_array_equal(run(bw, torch_cuda, parent, C, ev, qs),
                                  oracle_mod.ev_sweep(parent, C, ev, qs))


@pytest.mark.parametrize("shape", ["no_events", "no_queries", "single_state", "sparse_states"])
def test_degenerate_shapes(bw, torch_cuda, oracle_mod, shape):
    rng = np.random.default_rng(12)
    S, C, E, Q = 400, 300, 3000, 2000
    if shape == "single_state":
        S = 1
    parent = evgen.make_tree(S, "fork", rng)
    ev = evgen.make_events(S, C, 0 if shape == "no_events" else E, rng)
    qs = evgen.make_queries(S, C, 0 if shape == "no_queries" else Q, rng)
    if shape == "sparse_states":
        ev["state"] = (ev["state"] // 50) * 50
        qs["state"] = (qs["state"] // 37) * 37
    got = run(bw, torch_cuda, parent, C, ev, qs)
    np.testing.assert_array_equal(got, oracle_mod.ev_sweep(parent, C, ev, qs))


@pytest.mark.parametrize("bad", ["unsorted_events", "key_range", "query_range", "bad_parent",
                                 "unsorted_queries", "state_range"])
def test_rejected_inputs_report_status(bw, torch_cuda, bad):
    rng = np.random.default_rng(13)
    S, C = 300, 100
    parent = evgen.make_tree(S, "fork", rng)
    ev = evgen.make_events(S, C, 3000, rng)
    qs = evgen.make_queries(S, C, 1000, rng)
    if bad == "unsorted_events":
        ev["state"][10], ev["state"][2000] = ev["state"][2000], ev["state"][10]
    elif bad == "key_range":
        ev["key"][5] = C
    elif bad == "query_range":
        qs["hi"][3] = C + 1
    elif bad == "bad_parent":
        parent[17] = 40
    elif bad == "unsorted_queries":
        qs["state"][0] = S - 1
    elif bad == "state_range":
        ev["state"][-1] = S
    with pytest.raises(ValueError):
        run(bw, torch_cuda, parent, C, ev, qs)
    # the context stays usable after a rejected input
    ok = evgen.make_events(S, C, 100, rng)
    run(bw, torch_cuda, evgen.make_tree(S, "chain", rng), C, ok, evgen.make_queries(S, C, 10, rng))


@pytest.mark.parametrize("kind,blocks", [("fork", 0), ("chain", 3), ("star", 0)])
def test_heavy_states(bw, torch_cuda, oracle_mod, kind, blocks):
    """States with more events and more queries than one sweep tile stages, between
    ordinary states, on enter and exit steps."""
    rng = np.random.default_rng(21 + blocks)
    S, C = 600, 5000
    parent = evgen.make_tree(S, kind, rng)
    ecount = rng.poisson(3, S)
    qcount = rng.poisson(2, S)
    heavy = rng.choice(S, 12, replace=False)
    ecount[heavy] = rng.integers(800, 4000, heavy.size)
    qcount[heavy[:6]] = rng.integers(600, 2000, 6)
    ev = evgen.make_events(S, C, int(ecount.sum()), rng, zipf=1.1)
    ev["state"] = np.repeat(np.arange(S, dtype=np.uint32), ecount)
    qs = evgen.make_queries(S, C, int(qcount.sum()), rng)
    qs["state"] = np.repeat(np.arange(S, dtype=np.uint32), qcount)
    want = oracle_mod.ev_sweep(parent, C, ev, qs)
    np.testing.assert_array_equal(run(bw, torch_cuda, parent, C, ev, qs, blocks=blocks), want)
