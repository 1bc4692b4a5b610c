"""Multi-rank host path on CPU (gloo, two processes): every rank builds its own
seeded batch of trees (the bench's N > 1 sharding: independent trees, no exchange),
checks a sample of its answers with the oracle, and the bench's max-over-ranks
timing reduction returns the slowest rank's time on every rank."""
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
