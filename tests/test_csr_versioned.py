"""Config 3's versioned dimension: a chain-with-forks version tree over sparse u64
keys.  The keys' CSR rank index maps events and point/range lookups to ranks on the
device (bw_csr_events, bw_csr_queries) and the tree replays over the rank domain.
The oracle ranks on the host (np.searchsorted over the sorted distinct keys) and
replays with its preorder apply/undo checker."""
from __future__ import annotations

import numpy as np
import pytest


def oracle_ranks(w):
    keys = np.unique(w.ev_key)
    ev = np.empty(len(w.ev_key), dtype=[("state", "<u4"), ("key", "<u4"), ("delta", "<i8")])
    ev["state"], ev["key"], ev["delta"] = w.ev_state, np.searchsorted(keys, w.ev_key), w.ev_delta
    pt = np.empty(len(w.pt_key), dtype=[("state", "<u4"), ("lo", "<u4"), ("hi", "<u4")])
    r = np.searchsorted(keys, w.pt_key)
    present = (r < len(keys)) & (keys[np.minimum(r, len(keys) - 1)] == w.pt_key)
    pt["state"], pt["lo"], pt["hi"] = w.pt_state, np.where(present, r, 0), np.where(present, r + 1, 0)
    rg = np.empty(len(w.rg_lo), dtype=pt.dtype)
    rg["state"], rg["lo"], rg["hi"] = w.rg_state, np.searchsorted(keys, w.rg_lo), np.searchsorted(keys, w.rg_hi)
    return len(keys), ev, pt, rg


def test_versioned_workload_shape(bw):
    w = bw.workloads.csr_versioned(seed=3, scale=0.001)
    assert len(w.parent) == 100 and np.all(np.diff(w.ev_state.astype(np.int64)) >= 0)
    assert np.all(w.rg_lo <= w.rg_hi) and np.all(np.diff(w.pt_state.astype(np.int64)) >= 0)
    assert len(np.unique(w.ev_key)) == w.n_keys


@pytest.mark.gpu
@pytest.mark.parametrize("seed,scale", [(1, 0.002), (2, 0.01)])
def test_gpu_versioned_sparse_replay_matches_oracle(bw, torch_cuda, oracle_mod, seed, scale):
    import torch
    w = bw.workloads.csr_versioned(seed=seed, scale=scale)
    K, ev, pt, rg = oracle_ranks(w)
    want_pt = oracle_mod.ev_sweep(w.parent, K, ev, pt)
    want_rg = oracle_mod.ev_sweep(w.parent, K, ev, rg)
    dev = torch.device("cuda")

    def t(a, dtype):
        return torch.from_numpy(np.ascontiguousarray(a).view(dtype)).to(dev)
    p = torch.from_numpy(w.parent).to(dev)
    es, ek, ed = t(w.ev_state, np.int32), t(w.ev_key, np.int64), t(w.ev_delta, np.int64)
    got_pt, idx = bw.versioned_sparse_replay(p, es, ek, ed, t(w.pt_state, np.int32), t(w.pt_key, np.int64))
    assert idx.count() == K
    np.testing.assert_array_equal(got_pt.cpu().numpy(), want_pt)
    for path in ("auto", "general"):
        got_rg, _ = bw.versioned_sparse_replay(p, es, ek, ed, t(w.rg_state, np.int32), t(w.rg_lo, np.int64),
                                               t(w.rg_hi, np.int64), index=idx, path=path)
        np.testing.assert_array_equal(got_rg.cpu().numpy(), want_rg)
