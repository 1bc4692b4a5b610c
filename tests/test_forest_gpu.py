"""GPU parity of the batched forest replay (bw_forest_* through the C ABI) against
the oracle, tree by tree: uneven tree sizes and shapes, per-tree key domains,
trees without events or queries, one-state trees, many blocks per tree (multi-group
carry scans), CUDA-graph replays, the autotuner, and per-tree input errors."""
from __future__ import annotations

import numpy as np
import pytest

import evgen

pytestmark = pytest.mark.gpu

KINDS = ["chain", "bushy", "star", "fork"]


def make_forest(rng, T, max_states=3000, max_keys=70000, ev_per_state=6.0, q_per_tree=200, big=False):
    parents, events, queries, soff, eoff, qoff, keys = [], [], [], [0], [0], [0], []
    for t in range(T):
        S = int(rng.integers(1, max_states + 1)) if t % 7 else 1 + int(rng.integers(0, 3))
        C = int(rng.integers(1, max_keys + 1)) if t % 5 else int(rng.choice([1, 64, 65]))
        kind = KINDS[t % len(KINDS)]
        parents.append(evgen.make_tree(S, kind, rng, p_extend=0.95) if S > 1 else np.array([-1], np.int32))
        E = 0 if t % 11 == 3 else int(rng.poisson(ev_per_state * S))
        Q = 0 if t % 13 == 4 else int(rng.integers(1, q_per_tree + 1))
        events.append(evgen.make_events(S, C, E, rng, zipf=1.1 if t % 2 else 0.0, big=big))
        queries.append(evgen.make_queries(S, C, Q, rng))
        soff.append(soff[-1] + S); eoff.append(eoff[-1] + E); qoff.append(qoff[-1] + Q); keys.append(C)
    return (np.array(soff, np.int64), np.array(eoff, np.int64), np.array(qoff, np.int64),
            np.array(keys, np.uint32), np.concatenate(parents).astype(np.int32),
            np.concatenate(events), np.concatenate(queries))


def run_forest(bw, torch, F, tuning=None):
    soff, eoff, qoff, keys, par, ev, qs = F
    p, e, q = evgen.to_device(torch, par, ev, qs)
    return bw.forest_replay(soff, eoff, qoff, keys, p, e, q, tuning=tuning).cpu().numpy()


@pytest.mark.parametrize("seed,T,tuning", [
    (1, 40, None),
    (2, 120, None),
    (3, 30, {"block_work": 65536}),                     # many blocks per tree
    (4, 25, {"block_work": 20000, "ctas_per_sm": 1}),   # > 16 rows: two-pass carry scan
    (5, 60, {"slice_ranks": 512}),                       # several key slices per block
    (6, 50, {"tile": 1, "block_work": 65536}),           # narrow sweep tiles
    (7, 50, {"tile": 2, "ctas_per_sm": 1}),              # wide sweep tiles, one CTA per SM
    (8, 40, {"tile": 3}),                                # narrow tiles on 512 threads
    (9, 40, {"tile": 4, "block_work": 65536}),           # wide tiles on 512 threads
    (10, 40, {"tile": 5}),                               # one staging warp + 15 replay warps
    (13, 60, {"tile": 5, "block_work": 65536, "slice_ranks": 512}),
    (14, 60, {"tile": 6}),                               # Euler-tile sweep (bulk-copied signed tiles)
    (15, 40, {"tile": 6, "block_work": 65536}),
    (16, 60, {"tile": 6, "block_work": 65536, "slice_ranks": 512}),   # several slices per block
    (17, 25, {"tile": 6, "block_work": 20000}),          # > 16 carry rows per tree
    (18, 120, {"tile": 6, "slice_ranks": 2048}),
])
def test_forest_matches_oracle(bw, torch_cuda, oracle_mod, seed, T, tuning):
    rng = np.random.default_rng(seed)
    F = make_forest(rng, T)
    want = oracle_mod.ev_forest(*F)
    got = run_forest(bw, torch_cuda, F, tuning)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("tile", [0, 5, 6])
def test_forest_wrapping_deltas(bw, torch_cuda, oracle_mod, tile):
    rng = np.random.default_rng(11)
    F = make_forest(rng, 30, max_states=800, big=True)
    np.testing.assert_array_equal(run_forest(bw, torch_cuda, F, {"block_work": 40000, "tile": tile}),
                                  oracle_mod.ev_forest(*F))


@pytest.mark.parametrize("tile", [1, 2, 3, 4, 5, 6])
def test_forest_heavy_states_all_tiles(bw, torch_cuda, oracle_mod, tile):
    """States with more events and more queries than one sweep tile stages, in
    query-dense and query-sparse trees, under every tile geometry (single-probe and
    per-query-step replay, staged and direct reads)."""
    rng = np.random.default_rng(31 + tile)
    parents, events, queries, soff, eoff, qoff, keys = [], [], [], [0], [0], [0], []
    for t in range(6):
        S, C = int(rng.integers(200, 900)), int(rng.integers(500, 20000))
        parents.append(evgen.make_tree(S, KINDS[t % len(KINDS)], rng, p_extend=0.9))
        ecount = rng.poisson(4, S)
        qcount = rng.poisson(3.0 if t % 2 else 0.2, S)
        heavy = rng.choice(S, 4, replace=False)
        ecount[heavy] = rng.integers(600, 3000, heavy.size)
        qcount[heavy[:2]] = rng.integers(300, 1500, 2)
        ev = evgen.make_events(S, C, int(ecount.sum()), rng, zipf=1.1)
        ev["state"] = np.repeat(np.arange(S, dtype=np.uint32), ecount)
        qs = evgen.make_queries(S, C, int(qcount.sum()), rng)
        qs["state"] = np.repeat(np.arange(S, dtype=np.uint32), qcount)
        events.append(ev); queries.append(qs); keys.append(C)
        soff.append(soff[-1] + S); eoff.append(eoff[-1] + len(ev)); qoff.append(qoff[-1] + len(qs))
    F = (np.array(soff, np.int64), np.array(eoff, np.int64), np.array(qoff, np.int64),
         np.array(keys, np.uint32), np.concatenate(parents).astype(np.int32),
         np.concatenate(events), np.concatenate(queries))
    got = run_forest(bw, torch_cuda, F, {"tile": tile, "block_work": 30000})
    np.testing.assert_array_equal(got, oracle_mod.ev_forest(*F))


def test_unaligned_events_refused(bw, torch_cuda):
    """Events 8 but not 16 bytes aligned are refused on the host (both sweeps stage
    events with 16-byte copies): the launch fails with BW_EINVAL and nothing runs."""
    torch = torch_cuda
    rng = np.random.default_rng(19)
    soff, eoff, qoff, keys, par, ev, qs = make_forest(rng, 8, max_states=500)
    p, e, q = evgen.to_device(torch, par, ev, qs)
    buf = torch.empty(e.numel() + 1, dtype=torch.int64, device="cuda")
    e8 = buf[1:].view(-1, 2)          # 8-byte offset from a 256-byte-aligned base
    e8.copy_(e)
    assert e8.data_ptr() % 16 == 8
    for tuning in ({"tile": 6}, {"tile": 3}):
        with pytest.raises(RuntimeError):
            bw.forest_replay(soff, eoff, qoff, keys, p, e8, q, tuning=tuning)


def test_forest_equals_plain_per_tree(bw, torch_cuda):
    rng = np.random.default_rng(12)
    F = make_forest(rng, 16, max_states=2000)
    soff, eoff, qoff, keys, par, ev, qs = F
    got = run_forest(bw, torch_cuda, F)
    for t in range(len(keys)):
        s0, s1, e0, e1, q0, q1 = soff[t], soff[t + 1], eoff[t], eoff[t + 1], qoff[t], qoff[t + 1]
        p, e, q = evgen.to_device(torch_cuda, par[s0:s1], ev[e0:e1], qs[q0:q1])
        plain = bw.replay(p, int(keys[t]), e, q).cpu().numpy()
        np.testing.assert_array_equal(got[q0:q1], plain)


def test_forest_graph_replay_and_autotune(bw, torch_cuda, oracle_mod):
    torch = torch_cuda
    rng = np.random.default_rng(13)
    F = make_forest(rng, 64, max_states=4000)
    soff, eoff, qoff, keys, par, ev, qs = F
    want = oracle_mod.ev_forest(*F)
    p, e, q = evgen.to_device(torch, par, ev, qs)
    ans = torch.empty(len(qs), dtype=torch.int64, device="cuda")
    tuning, ms = bw.forest_autotune(soff, eoff, qoff, keys, p, e, q, ans, reps=2)
    assert ms > 0 and tuning["ctas_per_sm"] in (1, 2) and tuning["block_work"] > 0
    np.testing.assert_array_equal(ans.cpu().numpy(), want)
    f = bw.Forest(soff, eoff, qoff, keys, tuning=tuning)
    s = torch.cuda.Stream()
    ans.fill_(0)
    with torch.cuda.stream(s):
        f.capture(p, e, q, ans, s)
        for _ in range(3):
            f.replay(s)
    s.synchronize()
    assert f.status(s) == 0
    np.testing.assert_array_equal(ans.cpu().numpy(), want)
    info = f.info()
    assert info["blocks"] >= len(keys) and info["kernels"] > 10


@pytest.mark.parametrize("bad", ["parent", "key", "query", "state"])
def test_forest_rejects_bad_tree(bw, torch_cuda, bad):
    rng = np.random.default_rng(14)
    F = list(make_forest(rng, 12, max_states=300))
    soff, eoff, qoff, keys, par, ev, qs = F
    par, ev, qs = par.copy(), ev.copy(), qs.copy()
    t = 5
    if bad == "parent":
        par[soff[t] + soff[t + 1] - soff[t] - 1] = soff[t + 1] - soff[t] + 3   # parent beyond itself
        if soff[t + 1] - soff[t] == 1:
            par[soff[t]] = 0
        code = 5
    elif bad == "key":
        i = next(i for i in range(len(keys)) if eoff[i + 1] > eoff[i])
        ev["key"][eoff[i]] = keys[i]
        code = 2
    elif bad == "query":
        i = next(i for i in range(len(keys)) if qoff[i + 1] > qoff[i])
        qs["hi"][qoff[i]] = keys[i] + 1
        code = 4
    else:
        i = next(i for i in range(len(keys)) if eoff[i + 1] > eoff[i])
        ev["state"][eoff[i + 1] - 1] = soff[i + 1] - soff[i]
        code = 7
    p, e, q = evgen.to_device(torch_cuda, par, ev, qs)
    f = bw.Forest(soff, eoff, qoff, keys)
    ans = torch_cuda.empty(len(qs), dtype=torch_cuda.int64, device="cuda")
    f.launch(p, e, q, ans)
    assert f.status() == code


def test_forest_shape_errors(bw, torch_cuda):
    with pytest.raises(RuntimeError):
        bw.Forest([0, 0], [0, 0], [0, 0], [4])           # a tree without states
    with pytest.raises(RuntimeError):
        bw.Forest([0, 3], [0, 2], [0, 1], [0])           # empty key domain


@pytest.mark.parametrize("tuning", [None, {"tile": 3}, {"tile": 4, "block_work": 200000}, {"tile": 5},
                                    {"tile": 6}, {"tile": 6, "block_work": 200000}])
def test_one_tree_forest_equals_plain(bw, torch_cuda, tuning):
    """A forest of one tree is the plain replay (its uploaded tables, not the
    plain path's per-launch ones)."""
    rng = np.random.default_rng(15)
    S, C = 6000, 30000
    parent = evgen.make_tree(S, "fork", rng)
    ev = evgen.make_events(S, C, 150000, rng, zipf=1.1)
    qs = evgen.make_queries(S, C, 100000, rng)
    p, e, q = evgen.to_device(torch_cuda, parent, ev, qs)
    plain = bw.replay(p, C, e, q).cpu().numpy()
    got = bw.forest_replay([0, S], [0, len(ev)], [0, len(qs)], [C], p, e, q, tuning=tuning).cpu().numpy()
    np.testing.assert_array_equal(got, plain)


@pytest.mark.parametrize("chunks", [1, 3])
def test_host_forest_chunks(bw, torch_cuda, oracle_mod, chunks):
    """Replay from pinned host buffers in chunks of trees (copies overlapping the
    replay of other chunks), twice in a row, equals the oracle."""
    torch = torch_cuda
    rng = np.random.default_rng(16 + chunks)
    soff, eoff, qoff, keys, par, ev, qs = make_forest(rng, 30, max_states=2500)
    want = oracle_mod.ev_forest(soff, eoff, qoff, keys, par, ev, qs)
    hp = torch.from_numpy(par).pin_memory()
    he = torch.from_numpy(np.ascontiguousarray(ev).view(np.int64).reshape(-1, 2)).pin_memory()
    hq = torch.from_numpy(np.ascontiguousarray(qs).view(np.int32).reshape(-1, 3)).pin_memory()
    ha = torch.zeros(len(qs), dtype=torch.int64).pin_memory()
    hf = bw.HostForest(soff, eoff, qoff, keys, chunks=chunks)
    for _ in range(2):
        ha.zero_()
        hf.run(hp, he, hq, ha)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(ha.numpy(), want)
    assert hf.status() == 0 and len(hf.parts) == chunks
