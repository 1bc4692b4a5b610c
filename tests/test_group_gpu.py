"""Grouping ungrouped event and query arrays by state on the device
(bw_group_events, bw_group_queries): the result must equal a stable sort by state,
and a replay of the grouped arrays, its answers scattered back into input order,
must equal the oracle's answers for the original queries."""
from __future__ import annotations

import numpy as np
import pytest

import evgen

pytestmark = pytest.mark.gpu


# one radix pass (S <= 256), two (S <= 65,536: the query path's even case), three
@pytest.mark.parametrize("S,E,Q", [(200, 50_000, 3_000), (5_000, 80_000, 7_000), (70_000, 300_000, 40_000),
                                   (2, 1_000, 100), (1, 10, 3), (300_000, 100_000, 9_000), (40, 0, 0)])
def test_grouping_is_a_stable_sort(bw, torch_cuda, S, E, Q):
    import torch
    rng = np.random.default_rng(S + E)
    ev = evgen.make_events(S, 500, E, rng)
    qs = evgen.make_queries(S, 500, Q, rng)
    pe, pq = rng.permutation(E), rng.permutation(Q)
    ev_u, qs_u = ev[pe], qs[pq]
    _, e, q = evgen.to_device(torch_cuda, np.full(S, -1, np.int32), ev_u, qs_u)
    ge, gq, order = bw.group_by_state(S, e, q)
    want_e = ev_u[np.argsort(ev_u["state"], kind="stable")]
    want_o = np.argsort(qs_u["state"], kind="stable")
    np.testing.assert_array_equal(ge.cpu().numpy().view(want_e.dtype).reshape(-1), want_e)
    np.testing.assert_array_equal(gq.cpu().numpy().view(qs_u.dtype).reshape(-1), qs_u[want_o])
    np.testing.assert_array_equal(order.cpu().numpy(), want_o)


def test_grouped_replay_answers_in_input_order(bw, torch_cuda, oracle_mod):
    import torch
    rng = np.random.default_rng(3)
    S, C = 5_000, 1_024
    parent = evgen.make_tree(S, "fork", rng)
    ev = evgen.make_events(S, C, 200_000, rng)
    qs = evgen.make_queries(S, C, 30_000, rng)
    want = oracle_mod.ev_sweep(parent, C, ev, qs)
    pe, pq = rng.permutation(len(ev)), rng.permutation(len(qs))
    p, e, q = evgen.to_device(torch_cuda, parent, ev[pe], qs[pq])
    ge, gq, order = bw.group_by_state(S, e, q)
    ans = bw.replay(p, C, ge, gq)
    back = bw.scatter_device_answers(ans, order, len(qs)).cpu().numpy()   # input (shuffled) order
    np.testing.assert_array_equal(back, want[pq])


def test_grouping_reports_states_out_of_range(bw, torch_cuda):
    rng = np.random.default_rng(4)
    ev = evgen.make_events(100, 64, 5_000, rng)
    ev["state"][123] = 100
    _, e, _ = evgen.to_device(torch_cuda, np.full(100, -1, np.int32), ev, evgen.make_queries(100, 64, 1, rng))
    with pytest.raises(ValueError, match="state"):
        bw.group_by_state(100, e)
    ge, _, _ = bw.group_by_state(101, e)   # the context stays usable
    assert ge.shape == e.shape
