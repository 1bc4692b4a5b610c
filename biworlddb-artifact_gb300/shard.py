"""One version chain split across ranks (one process per GPU).

A chain's events grouped by state are its replay order, so rank r takes the
contiguous state range [s_r, s_{r+1}) -- its events and the queries at those states,
with states renumbered from 0 -- and replays it alone as a chain of its own.  What
the rank does not see is the carry: the dense key histogram of every event below
s_r.  It is the only exchange: an exclusive scan over ranks of each rank's own
histogram (n_keys int64), the reference's serial carry pass
(batch_engine_v7.hpp:936-945) lifted from state blocks to ranks.  Each rank then
adds the carry inside [lo, hi) to its answers, as the reference's combine does
(batch_engine_v7.hpp:948-961).  Queries stay local; answers come out in the global
query order when the ranks' slices are concatenated.

``Exchange`` is the interface of that one collective.  ``LocalExchange`` is the
one-rank form (the identity: nothing below rank 0); ``DistExchange`` runs over an
initialised torch.distributed process group (NCCL between GPUs, gloo on CPU);
``split_chain`` cuts the ranks' state ranges at state boundaries with about equal
events; ``ShardedChain`` drives one rank with a pluggable engine -- ``GpuEngine``
(the CUDA replay plus bw_key_histogram / bw_key_prefix / bw_add_range_carry) in
the product.
"""
from __future__ import annotations

import numpy as np

M64 = (1 << 64) - 1


class Exchange:
    """The carry collective: given this rank's int64 vector, return the wrapping sum of
    the vectors of every lower rank (an exclusive scan over ranks)."""

    rank = 0
    world = 1

    def exclusive_scan(self, vec: np.ndarray) -> np.ndarray:
        raise NotImplementedError


class LocalExchange(Exchange):
    """One rank: nothing lies below it."""

    def exclusive_scan(self, vec: np.ndarray) -> np.ndarray:
        return np.zeros_like(np.asarray(vec, dtype=np.int64))


class DistExchange(Exchange):
    """Exclusive scan over the ranks of an initialised torch.distributed group: an
    all-gather of the int64 vectors, then the wrapping sum of the lower ranks'."""

    def __init__(self, group=None, device=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        self.device = device

    def exclusive_scan(self, vec: np.ndarray) -> np.ndarray:
        import torch
        v = np.ascontiguousarray(vec, dtype=np.int64)
        t = torch.from_numpy(v.copy())
        if self.device is not None:
            t = t.to(self.device)
        parts = [torch.empty_like(t) for _ in range(self.world)]
        self.dist.all_gather(parts, t, group=self.group)
        acc = np.zeros(v.size, dtype=np.uint64)
        for r in range(self.rank):
            acc += parts[r].cpu().numpy().view(np.uint64)
        return acc.view(np.int64)


def split_chain(event_state: np.ndarray, n_states: int, world: int) -> list[tuple[int, int]]:
    """State ranges [s_r, s_{r+1}) of `world` ranks, cut at state boundaries so every
    rank holds about the same number of events (every rank gets at least one state)."""
    E = int(event_state.size)
    if world < 1 or n_states < world:
        raise ValueError("need at least one state per rank")
    cuts = [0]
    for r in range(1, world):
        s = int(event_state[min(E - 1, E * r // world)]) if E else n_states * r // world
        s = max(s, cuts[-1] + 1)
        s = min(s, n_states - (world - r))
        cuts.append(s)
    cuts.append(n_states)
    return list(zip(cuts[:-1], cuts[1:]))


def shard_inputs(parent, events, queries, s0: int, s1: int):
    """Rank-local inputs of the state range [s0, s1): a chain of s1 - s0 states, the
    range's events and queries with states renumbered from 0, and the range's
    positions in the global event and query arrays."""
    ev_st = events["state"]
    q_st = queries["state"]
    e0, e1 = int(np.searchsorted(ev_st, s0, "left")), int(np.searchsorted(ev_st, s1, "left"))
    q0, q1 = int(np.searchsorted(q_st, s0, "left")), int(np.searchsorted(q_st, s1, "left"))
    n = s1 - s0
    par = (np.arange(n, dtype=np.int64) - 1).astype(np.int32)
    ev = events[e0:e1].copy()
    ev["state"] -= np.uint32(s0)
    qs = queries[q0:q1].copy()
    qs["state"] -= np.uint32(s0)
    return par, ev, qs, (e0, e1), (q0, q1)


class GpuEngine:
    """The CUDA side of one rank: chain replay, key histogram, carry fix-up."""

    def __init__(self, bw, device=None):
        import torch
        self.bw = bw
        self.torch = torch
        self.device = device or torch.device("cuda", torch.cuda.current_device())

    def replay(self, parent, n_keys, events, queries):
        torch, bw = self.torch, self.bw
        self.d_par = torch.from_numpy(np.ascontiguousarray(parent)).to(self.device)
        self.d_ev = torch.from_numpy(np.ascontiguousarray(events).view(np.int64).reshape(-1, 2)).to(self.device)
        self.d_q = torch.from_numpy(np.ascontiguousarray(queries).view(np.int32).reshape(-1, 3)).to(self.device)
        self.ans = bw.replay(self.d_par, n_keys, self.d_ev, self.d_q, chain=True)
        return self.ans

    def histogram(self, n_keys, events):
        import ctypes as C
        torch, L = self.torch, self.bw.gpu_lib()
        L.bw_key_histogram.argtypes = [C.c_void_p, C.c_int64, C.c_uint32, C.c_void_p, C.c_void_p]
        h = torch.empty(n_keys, dtype=torch.int64, device=self.device)
        n = int(self.d_ev.shape[0])
        st = torch.cuda.current_stream(self.device).cuda_stream
        self.bw._check(L.bw_key_histogram(self.d_ev.data_ptr() if n else None, n, n_keys, h.data_ptr(), st),
                       "bw_key_histogram")
        return h.cpu().numpy()

    def add_carry(self, n_keys, queries, carry):
        import ctypes as C
        torch, L = self.torch, self.bw.gpu_lib()
        L.bw_key_prefix.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
        L.bw_add_range_carry.argtypes = [C.c_void_p, C.c_int64, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
        st = torch.cuda.current_stream(self.device).cuda_stream
        d_carry = torch.from_numpy(np.ascontiguousarray(carry, dtype=np.int64)).to(self.device)
        prefix = torch.empty(n_keys + 1, dtype=torch.int64, device=self.device)
        self.bw._check(L.bw_key_prefix(d_carry.data_ptr(), n_keys, prefix.data_ptr(), st), "bw_key_prefix")
        n = int(self.d_q.shape[0])
        self.bw._check(L.bw_add_range_carry(self.d_q.data_ptr() if n else None, n, n_keys, prefix.data_ptr(),
                                            self.ans.data_ptr() if n else None, st), "bw_add_range_carry")
        return self.ans.cpu().numpy()


class ShardedChain:
    """One rank's part of a chain replay split over `exchange.world` ranks."""

    def __init__(self, exchange: Exchange, engine):
        self.ex = exchange
        self.engine = engine

    def run(self, parent, n_keys: int, events, queries):
        """This rank's answers (the global queries of its state range, in order) and
        the range's global query positions (q0, q1)."""
        cuts = split_chain(events["state"], int(len(parent)), self.ex.world)
        s0, s1 = cuts[self.ex.rank]
        par, ev, qs, _, qrange = shard_inputs(parent, events, queries, s0, s1)
        self.engine.replay(par, n_keys, ev, qs)
        hist = self.engine.histogram(n_keys, ev)
        carry = self.ex.exclusive_scan(hist)
        return self.engine.add_carry(n_keys, qs, carry), qrange
