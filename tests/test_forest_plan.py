"""Host-side forest planning on CPU (bw_forest_plan_stats, no GPU): every tree
gets at least one block, a smaller block work never gives fewer blocks, the dense
carry rows stay within the 4 GB budget for every tuning, one-block trees need no
carry, and malformed shapes are refused."""
from __future__ import annotations

import numpy as np
import pytest


@pytest.fixture(scope="module")
def forest(bw):
    return bw.workloads.batched_trees(seed=1, trees=300, median=1500, cap=60000, queries_per_tree=200)


def args(w):
    return (w.state_off, w.event_off, w.query_off, w.n_keys)


def test_every_tree_has_a_block(bw, forest):
    st = bw.forest_plan_stats(*args(forest), tuning={"block_work": 1 << 40})
    assert st["blocks"] == forest.n_trees and st["carry_bytes"] == 0


@pytest.mark.parametrize("tile", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("ctas", [1, 2])
def test_block_work_monotone_and_carry_budget(bw, forest, tile, ctas):
    prev = None
    for bwk in [1 << 26, 1 << 22, 1 << 19, 65536]:
        st = bw.forest_plan_stats(*args(forest), tuning={"block_work": bwk, "tile": tile, "ctas_per_sm": ctas})
        assert st["carry_bytes"] <= 4e9 and st["workspace_bytes"] > 0
        if prev is not None:
            assert st["blocks"] >= prev
        prev = st["blocks"]


def test_carry_budget_caps_huge_domains(bw):
    # two big trees on 2^28-key domains: tiny blocks would need > 4 GB of carry rows
    soff, eoff, qoff = np.array([0, 50000, 100000]), np.array([0, 800000, 1600000]), np.array([0, 100, 200])
    st = bw.forest_plan_stats(soff, eoff, qoff, np.array([1 << 28, 1 << 28], np.uint32), tuning={"block_work": 65536})
    assert st["carry_bytes"] <= 4e9 and st["blocks"] >= 2


def test_unknown_tile_refused(bw, forest):
    with pytest.raises(RuntimeError):
        bw.forest_plan_stats(*args(forest), tuning={"tile": 7})


def test_malformed_shapes_refused(bw):
    with pytest.raises(RuntimeError):
        bw.forest_plan_stats([0, 0], [0, 0], [0, 0], [4])          # a tree without states
    with pytest.raises(RuntimeError):
        bw.forest_plan_stats([0, 3], [0, 2], [0, 1], [0])          # empty key domain
    with pytest.raises(RuntimeError):
        bw.forest_plan_stats([0, 3, 5], [0, 4, 2], [0, 1, 1], [4, 4])   # event offsets decrease
