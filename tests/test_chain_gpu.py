"""GPU parity of the single-pass chain path (csrc/bw_chain.cu) against the oracle.

The chain path takes event-heavy chains with key domains up to 32,768 keys: each
event is read once through bulk-copied shared-memory tiles, the block histogram
is kept in exact int32 windows flushed into int64 rows, and tiles with large
deltas go straight to the int64 rows.  The cases cover every branch of that
scheme: small deltas (window only), medium deltas (window flushes every few
tiles), huge and wrapping deltas (wide tiles), mixed tiles, one block and many
forced blocks, tiny and maximal key domains, no events, no queries, queries
before the first event and after the last, many queries on one state (more than
a tile stages), empty/reversed/full intervals, and the device-side input checks.
Each case asserts the chain path was the one taken."""
from __future__ import annotations

import numpy as np
import pytest

import evgen

pytestmark = pytest.mark.gpu


def chain_case(seed, S, C, E, Q, zipf=1.1, delta="small"):
    rng = np.random.default_rng(seed)
    parent = evgen.make_tree(S, "chain", rng)
    ev = evgen.make_events(S, C, E, rng, zipf=zipf, big=(delta == "huge"))
    if delta == "medium":     # ~2^17 per event: the int32 window fills within a few tiles
        ev["delta"] = rng.integers(-(1 << 17), 1 << 17, E)
    elif delta == "mixed":    # mostly small, a few tiles carry one 2^40 delta
        hot = rng.random(E) < 2e-4
        ev["delta"][hot] = rng.integers(-(1 << 40), 1 << 40, int(hot.sum()))
    qs = evgen.make_queries(S, C, Q, rng)
    return parent, C, ev, qs


def run_chain(bw, torch, parent, C, ev, qs, blocks=0, path="chain", wide=False):
    p, e, q = evgen.to_device(torch, parent, ev, qs)
    r = bw.Replay(p, C, len(ev), len(qs), blocks=blocks, chain=True, path=path, wide=wide)
    assert r.chain_path(e), "the chain path was not selected"
    ans = torch.empty(len(qs), dtype=torch.int64, device=p.device)
    r.launch(p, e, q, ans)
    st = r.status()
    return ans.cpu().numpy(), st


CASES = [
    # seed, S, C, E, Q, zipf, delta, blocks
    (1, 20000, 4096, 1_000_000, 10_000, 1.1, "small", 0),      # the plain-chain shape, scaled down
    (2, 20000, 4096, 1_000_000, 10_000, 1.1, "small", 1),
    (3, 5000, 4096, 300_000, 30_000, 1.1, "medium", 0),
    (4, 5000, 4096, 300_000, 30_000, 1.1, "medium", 3),
    (5, 3000, 1000, 200_000, 20_000, 0.0, "huge", 0),
    (6, 3000, 1000, 200_000, 20_000, 0.0, "mixed", 5),
    (7, 4000, 32768, 400_000, 40_000, 1.2, "small", 0),
    (8, 4000, 32768, 400_000, 40_000, 0.0, "mixed", 0),
    (9, 200, 1, 50_000, 3_000, 0.0, "small", 0),
    (10, 900, 37, 70_000, 8_000, 0.0, "medium", 17),
    (11, 100_000, 64, 500_000, 60_000, 0.0, "small", 0),     # more states than events per block
    (12, 2, 300, 40_000, 5_000, 0.0, "small", 0),            # two states
]


@pytest.mark.parametrize("seed,S,C,E,Q,zipf,delta,blocks", CASES)
def test_chain_path_matches_oracle(bw, torch_cuda, oracle_mod, seed, S, C, E, Q, zipf, delta, blocks):
    parent, C, ev, qs = chain_case(seed, S, C, E, Q, zipf, delta)
    want = oracle_mod.ev_blocks(parent, C, ev, qs, blocks=8)
    got, st = run_chain(bw, torch_cuda, parent, C, ev, qs, blocks=blocks)
    assert st == 0
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("seed,S,C,E,Q,zipf,delta,blocks", [c for c in CASES if c[2] <= 16384])
def test_chain_path_int64_window_matches_oracle(bw, torch_cuda, oracle_mod, seed, S, C, E, Q, zipf, delta, blocks):
    """BW_REPLAY_WIDE: the same cases through the int64 histogram (any delta size,
    no window folds, no wide tiles)."""
    parent, C, ev, qs = chain_case(seed, S, C, E, Q, zipf, delta)
    want = oracle_mod.ev_blocks(parent, C, ev, qs, blocks=8)
    got, st = run_chain(bw, torch_cuda, parent, C, ev, qs, blocks=blocks, wide=True)
    assert st == 0
    np.testing.assert_array_equal(got, want)


def test_chain_path_many_blocks_equal_general_path(bw, torch_cuda, oracle_mod):
    parent, C, ev, qs = chain_case(20, 30000, 2048, 600_000, 70_000)
    want = oracle_mod.ev_blocks(parent, C, ev, qs, blocks=8)
    for blocks in (2, 31, 300, 1200):
        got, st = run_chain(bw, torch_cuda, parent, C, ev, qs, blocks=blocks)
        assert st == 0
        np.testing.assert_array_equal(got, want)
    p, e, q = evgen.to_device(torch_cuda, parent, ev, qs)
    np.testing.assert_array_equal(bw.replay(p, C, e, q, chain=True, path="general").cpu().numpy(), want)


def test_chain_path_edge_shapes(bw, torch_cuda, oracle_mod):
    rng = np.random.default_rng(30)
    S, C = 6000, 512
    parent = evgen.make_tree(S, "chain", rng)
    # events only on a middle band of states; queries before, inside and after it,
    # with 500 queries on a single state (more than one tile stages)
    ev = evgen.make_events(S, C, 120_000, rng)
    ev["state"] = np.sort(rng.integers(2000, 4000, len(ev))).astype(np.uint32)
    qs = evgen.make_queries(S, C, 20_000, rng)
    qs["state"][:500] = 3000
    qs = qs[np.argsort(qs["state"], kind="stable")]
    want = oracle_mod.ev_sweep(parent, C, ev, qs)
    for blocks in (0, 1, 9):
        got, st = run_chain(bw, torch_cuda, parent, C, ev, qs, blocks=blocks)
        assert st == 0
        np.testing.assert_array_equal(got, want)
    # no events: every answer is 0
    empty = ev[:0]
    got, st = run_chain(bw, torch_cuda, parent, C, empty, qs)
    assert st == 0 and not got.any()
    # no queries
    got, st = run_chain(bw, torch_cuda, parent, C, ev, qs[:0])
    assert st == 0 and got.size == 0


@pytest.mark.parametrize("defect,code", [("events_unsorted", 1), ("event_key", 2), ("queries_unsorted", 3),
                                         ("query_bound", 4), ("fork", 5), ("query_state", 7)])
def test_chain_path_reports_bad_input(bw, torch_cuda, defect, code):
    parent, C, ev, qs = chain_case(40, 3000, 1024, 200_000, 20_000)
    ev, qs, parent = ev.copy(), qs.copy(), parent.copy()
    if defect == "events_unsorted":
        ev["state"][100_000] = ev["state"][-1]
    elif defect == "event_key":
        ev["key"][12345] = C + 7
    elif defect == "queries_unsorted":
        qs["state"][5000] = qs["state"][-1]
    elif defect == "query_bound":
        qs["hi"][777] = C + 1
    elif defect == "fork":
        parent[1500] = 10
    elif defect == "query_state":
        qs["state"][-1] = 3000
    _, st = run_chain(bw, torch_cuda, parent, C, ev, qs)
    assert st == code
    # the context stays usable
    parent, C, ev, qs = chain_case(41, 300, 64, 20_000, 2_000)
    got, st = run_chain(bw, torch_cuda, parent, C, ev, qs)
    assert st == 0


def test_chain_path_selection(bw, torch_cuda):
    """Auto selection: event-heavy chains with small domains take the chain path;
    query-heavy ones, large domains, trees and forced-general runs do not."""
    import torch
    dev = torch.device("cuda")
    p = torch.zeros(100, dtype=torch.int32, device=dev)
    e = torch.zeros((8000, 2), dtype=torch.int64, device=dev)
    assert bw.Replay(p, 4096, 8000, 1000, chain=True).chain_path(e)
    assert not bw.Replay(p, 4096, 8000, 1001, chain=True).chain_path(e)
    assert bw.Replay(p, 4096, 8000, 5000, chain=True, path="chain").chain_path(e)
    assert not bw.Replay(p, 40000, 8000, 1000, chain=True).chain_path(e)
    assert not bw.Replay(p, 4096, 8000, 1000, chain=False).chain_path(e)
    assert not bw.Replay(p, 4096, 8000, 1000, chain=True, path="general").chain_path(e)
    # events not 16-byte aligned: not the chain path (a launch refuses them: BW_EINVAL)
    e2 = torch.zeros(16002, dtype=torch.int64, device=dev)[1:16001].view(-1, 2)
    assert not bw.Replay(p, 4096, 8000, 1000, chain=True).chain_path(e2)
