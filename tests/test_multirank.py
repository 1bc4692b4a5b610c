"""Multi-rank host paths on CPU (gloo, separate processes).

* Batched trees (the bench's N > 1 sharding): every rank builds its own seeded batch
  of trees (independent trees, no exchange), checks its answers with the oracle, and
  the bench's max-over-ranks timing reduction returns the slowest rank's time.
* One chain split over ranks (shard.py): each rank runs the repository's own split
  (split_chain, shard_inputs), its exchange (DistExchange: the exclusive scan of the
  ranks' key histograms over torch.distributed) and the carry fix-up, with a CPU
  restatement of the three device steps standing in for the GPU (the oracle's block
  executor for the local replay, numpy for bw_key_histogram, bw_key_prefix and
  bw_add_range_carry); the concatenated answers must equal the one-rank oracle.
  On hardware this path is unmeasured: every run here has one GPU."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _rank_main(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    sys.path.insert(0, str(ROOT / "oracle"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        import oracle
        from conftest import load_package
        bw = load_package()
        w = bw.workloads.batched_trees(seed=rank, trees=12, median=200, cap=2000, queries_per_tree=40)
        ans = oracle.ev_forest(w.state_off, w.event_off, w.query_off, w.n_keys, w.parent, w.events, w.queries)
        brute = oracle.ev_forest(w.state_off, w.event_off, w.query_off, w.n_keys, w.parent, w.events, w.queries,
                                 fn=lambda p, C, e, q: oracle.ev_bruteforce(p, e, q))
        ok = bool(np.array_equal(ans, brute))
        ms = bench.max_over_ranks(1.0 + rank, "cpu")
        dist.barrier()
        out.put((rank, ok, ms, oracle.sha256_hex(ans.tobytes())))
    finally:
        dist.destroy_process_group()


def test_two_rank_sharded_batches_and_timing():
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert all(ok for _, ok, _, _ in res)
    assert all(ms == 2.0 for _, _, ms, _ in res)          # the slowest rank's time everywhere
    assert res[0][3] != res[1][3]                            # each rank has its own batch


class CpuEngine:
    """CPU restatement of shard.GpuEngine's three device steps (test double)."""

    def __init__(self, oracle):
        self.oracle = oracle

    def replay(self, parent, n_keys, events, queries):
        self.ans = self.oracle.ev_blocks(parent, n_keys, events, queries, blocks=3, threads=1)
        return self.ans

    def histogram(self, n_keys, events):
        h = np.zeros(n_keys, dtype=np.uint64)
        keep = events["key"] < n_keys
        np.add.at(h, events["key"][keep].astype(np.int64), events["delta"][keep].view(np.uint64))
        return h.view(np.int64)

    def add_carry(self, n_keys, queries, carry):
        pre = np.concatenate([[np.uint64(0)], np.cumsum(np.asarray(carry).view(np.uint64), dtype=np.uint64)])
        lo = np.minimum(queries["lo"], n_keys).astype(np.int64)
        hi = np.minimum(queries["hi"], n_keys).astype(np.int64)
        m = lo < hi
        out = self.ans.view(np.uint64).copy()
        out[m] += pre[hi[m]] - pre[lo[m]]
        return out.view(np.int64)


def _chain(seed):
    import evgen
    rng = np.random.default_rng(seed)
    S, C = 4000, 777
    parent = evgen.make_tree(S, "chain", rng)
    ev = evgen.make_events(S, C, 60000, rng, zipf=1.1, big=seed % 2 == 1)
    qs = evgen.make_queries(S, C, 20000, rng)
    return parent, C, ev, qs


def _shard_rank_main(rank: int, world: int, port: int, seed: int, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    sys.path.insert(0, str(ROOT / "oracle"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        from conftest import load_package
        bw = load_package()
        parent, C, ev, qs = _chain(seed)
        sc = bw.shard.ShardedChain(bw.shard.DistExchange(), CpuEngine(oracle))
        ans, (q0, q1) = sc.run(parent, C, ev, qs)
        dist.barrier()
        out.put((rank, q0, q1, ans.tobytes()))
    finally:
        dist.destroy_process_group()


def _spawn(target, world, extra):
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=target, args=(r, world, port, *extra, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=180) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return sorted(res)


@pytest.mark.parametrize("world,seed", [(2, 0), (3, 1)])
def test_chain_split_over_ranks_equals_one_rank(oracle_mod, world, seed):
    res = _spawn(_shard_rank_main, world, (seed,))
    parent, C, ev, qs = _chain(seed)
    want = oracle_mod.ev_sweep(parent, C, ev, qs)
    got = np.zeros(len(qs), dtype=np.int64)
    covered = 0
    for _, q0, q1, buf in res:
        got[q0:q1] = np.frombuffer(buf, dtype=np.int64)
        covered += q1 - q0
    assert covered == len(qs)
    np.testing.assert_array_equal(got, want)


def test_split_chain_cuts_balance_events_at_state_boundaries(bw):
    parent, C, ev, qs = _chain(4)
    for world in (1, 2, 5, 16):
        cuts = bw.shard.split_chain(ev["state"], len(parent), world)
        assert cuts[0][0] == 0 and cuts[-1][1] == len(parent) and len(cuts) == world
        assert all(a < b for a, b in cuts) and all(cuts[i][1] == cuts[i + 1][0] for i in range(world - 1))
        counts = [int(np.sum((ev["state"] >= a) & (ev["state"] < b))) for a, b in cuts]
        assert max(counts) <= len(ev) / world + 200   # events of one state at most off
    assert bw.shard.LocalExchange().exclusive_scan(np.arange(5)).tolist() == [0] * 5
