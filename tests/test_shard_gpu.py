"""GPU side of one chain split over ranks (shard.py, csrc/bw_shard.cu).

Every run here has one GPU, so ranks are not run concurrently: a one-rank run
(LocalExchange, the identity form) and several ranks run one after another in this
process, each with its own device buffers, through an exchange double that hands
rank r the sum of the histograms ranks 0..r-1 produced (no kernel waits on another).
The concatenated answers must equal the oracle's; the device histogram, key prefix
and carry fix-up are also checked against numpy on their own."""
from __future__ import annotations

import numpy as np
import pytest

import evgen

pytestmark = pytest.mark.gpu


class SequentialExchange:
    """Ranks 0..world-1 call exclusive_scan in order within one process."""

    def __init__(self, world):
        self.world, self.rank, self.sums = world, 0, np.zeros(0, dtype=np.uint64)

    def exclusive_scan(self, vec):
        v = np.asarray(vec, dtype=np.int64).view(np.uint64)
        if self.sums.size == 0:
            self.sums = np.zeros(v.size, dtype=np.uint64)
        out = self.sums.copy()
        self.sums = self.sums + v
        return out.view(np.int64)


def chain(seed, S=6000, C=2048, E=300_000, Q=40_000, big=False):
    rng = np.random.default_rng(seed)
    return (evgen.make_tree(S, "chain", rng), C, evgen.make_events(S, C, E, rng, zipf=1.1, big=big),
            evgen.make_queries(S, C, Q, rng))


@pytest.mark.parametrize("world,big", [(1, False), (3, False), (4, True)])
def test_chain_split_on_one_gpu_equals_oracle(bw, torch_cuda, oracle_mod, world, big):
    parent, C, ev, qs = chain(50 + world, big=big)
    want = oracle_mod.ev_sweep(parent, C, ev, qs)
    got = np.zeros(len(qs), dtype=np.int64)
    ex = bw.shard.LocalExchange() if world == 1 else SequentialExchange(world)
    for r in range(world):
        ex.rank = r
        ex.world = world
        sc = bw.shard.ShardedChain(ex, bw.shard.GpuEngine(bw))
        ans, (q0, q1) = sc.run(parent, C, ev, qs)
        got[q0:q1] = ans
    np.testing.assert_array_equal(got, want)


def test_histogram_prefix_and_carry_kernels(bw, torch_cuda):
    rng = np.random.default_rng(9)
    for C in (5, 4096, 40000):            # shared-memory and global histogram forms
        ev = evgen.make_events(100, C, 200_000, rng, zipf=1.2, big=C == 5)
        qs = evgen.make_queries(100, C, 30_000, rng)
        eng = bw.shard.GpuEngine(bw)
        eng.replay(evgen.make_tree(100, "chain", rng), C, ev, qs)
        h = eng.histogram(C, ev)
        want_h = np.zeros(C, dtype=np.uint64)
        np.add.at(want_h, ev["key"].astype(np.int64), ev["delta"].view(np.uint64))
        np.testing.assert_array_equal(h.view(np.uint64), want_h)
        base = eng.ans.cpu().numpy().view(np.uint64).copy()
        carry = rng.integers(-2**62, 2**62, C, dtype=np.int64)
        got = eng.add_carry(C, qs, carry).view(np.uint64)
        pre = np.concatenate([[np.uint64(0)], np.cumsum(carry.view(np.uint64), dtype=np.uint64)])
        lo = np.minimum(qs["lo"], C).astype(np.int64)
        hi = np.minimum(qs["hi"], C).astype(np.int64)
        m = lo < hi
        base[m] += pre[hi[m]] - pre[lo[m]]
        np.testing.assert_array_equal(got, base)
