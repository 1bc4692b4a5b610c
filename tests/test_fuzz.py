"""Randomized branching fuzz through the GPU path.

The reference's fuzz harness (fuzz_fullpath.cpp) draws tiny fixtures and declared
workloads over 10 profiles (row-heavy, factor-heavy, forced empty ranges, inserts
at t_max+1, negative amounts, factor edits to 0, negative factors, all-factor, a
dense 8-tick frame, mixed), 3 topologies (chain, bushy, star) and both range scopes
(per-state and shared), the first 60 cases being the deterministic edge cases.  It
checks its arms against a rollback-Fenwick oracle but never runs the v7 executor or
any GPU kernel (fuzz_fullpath.cpp:38-44).  Here every case runs through the host
front end (bw_native_build_declared) and the CUDA replay (bw_replay_launch: the
general pipeline with and without the chain hint and with forced state blocks, and
for chains the single-pass chain path too), chains also through the gpu_v7.h
drop-in (gpu_v7_launch + carry + gpu_combine_launch), and every answer vector must
hash to the value the reference's own build_case + "rf" arm produced
(tests/golden/fuzz_golden.json, made by make_fuzz_golden.py).
"""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import fuzzgen

GOLD = json.loads((Path(__file__).resolve().parent / "golden" / "fuzz_golden.json").read_text())
CHUNK = 75
RUNS = {r["states"]: r["cases"] for r in GOLD["runs"]}
CHUNKS = [(states, i) for states, cases in RUNS.items() for i in range(0, len(cases), CHUNK)]


def chunk_id(c):
    return f"S{c[0]}-cases{c[1]}"


def cases_of(chunk):
    states, i = chunk
    for rec in RUNS[states][i:i + CHUNK]:
        yield rec, fuzzgen.case(rec["case"], states)


def test_fuzz_coverage():
    """The golden set spans every profile, topology and range scope, and the edge
    values the reference fuzz targets."""
    seen = {"profile": set(), "topology": set(), "scope": set()}
    zero_f = neg_f = tmax1 = empty = neg_amt = 0
    for states, cases in RUNS.items():
        for rec in cases:
            c = fuzzgen.case(rec["case"], states)
            seen["profile"].add(c.profile)
            seen["topology"].add(c.topology)
            seen["scope"].add(c.per_state)
            f = c.op == fuzzgen.OP_FACTOR
            zero_f += int(np.sum(f & (c.val == 0)))
            neg_f += int(np.sum(f & (c.val < 0)))
            tmax1 += int(np.sum(np.isin(c.op, (fuzzgen.OP_INSERT, fuzzgen.OP_MOVE)) & (c.t > 1000008) & (c.profile == 3)))
            empty += int(np.sum(c.qlo == c.qhi))
            if c.profile == 4:
                neg_amt += 1
    assert seen == {"profile": set(range(10)), "topology": {0, 1, 2}, "scope": {True, False}}
    assert min(zero_f, neg_f, tmax1, empty, neg_amt) > 0
    assert sum(len(c) for c in RUNS.values()) >= 300


@pytest.mark.parametrize("chunk", CHUNKS, ids=chunk_id)
def test_fuzz_generator_matches_reference(chunk):
    for rec, c in cases_of(chunk):
        assert hashlib.sha256(c.fixture).hexdigest() == rec["fixture_sha256"], c.name
        assert (c.seed, c.profile, c.topology, c.q, c.per_state, c.N, c.G, c.p_factor) == (
            rec["seed"], rec["profile"], rec["topology"], rec["q"], rec["per_state"], rec["N"], rec["G"],
            rec["p_factor"]), c.name


@pytest.mark.parametrize("chunk", CHUNKS, ids=chunk_id)
def test_fuzz_oracle_matches_reference(oracle_mod, chunk):
    for rec, c in cases_of(chunk):
        ans = oracle_mod.direct_scan_declared(oracle_mod.Fixture(c.fixture), c)
        assert ans.size == rec["n_answers"]
        assert oracle_mod.sha256_hex(ans.tobytes()) == rec["answers_sha256"], c.name


@pytest.mark.parametrize("chunk", CHUNKS, ids=chunk_id)
def test_fuzz_front_end_matches_reference(bw, oracle_mod, chunk):
    import v7_emul
    for rec, c in cases_of(chunk):
        w = bw.native_workload_declared(c.fixture, c, c.name)
        ans = oracle_mod.ev_sweep(w.parent, w.n_keys, w.events, w.queries)
        assert bw.sha256_hex(ans.tobytes()) == rec["answers_sha256"], c.name
        if w.chain:
            plan = bw.v7_plan_declared(c.fixture, c, 4)
            got, _, _ = v7_emul.run(plan)
            assert bw.sha256_hex(got.tobytes()) == rec["answers_sha256"], c.name


def test_declared_front_end_rejects_bad_edits(bw):
    c = fuzzgen.case(9, 33)
    bad = fuzzgen.case(9, 33)
    bad.op = c.op.copy()
    bad.op[5] = 9
    with pytest.raises(ValueError):
        bw.native_workload_declared(bad.fixture, bad)
    bad = fuzzgen.case(9, 33)
    i = int(np.nonzero(bad.op != fuzzgen.OP_FACTOR)[0][1])
    bad.id = c.id.copy()
    bad.id[i] = c.N + len(c.ins_t) + 5
    with pytest.raises(ValueError):
        bw.native_workload_declared(bad.fixture, bad)
    bad = fuzzgen.case(9, 33)
    bad.parent = c.parent.copy()
    bad.parent[4] = 9
    with pytest.raises(ValueError):
        bw.native_workload_declared(bad.fixture, bad)
    tree = fuzzgen.case(13, 33)   # bushy: no v7 chain plan
    assert tree.topology == 1
    with pytest.raises(ValueError):
        bw.v7_plan_declared(tree.fixture, tree, 2)


# ------------------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("chunk", CHUNKS, ids=chunk_id)
def test_gpu_fuzz_replay(bw, torch_cuda, chunk):
    import evgen
    n = 0
    for rec, c in cases_of(chunk):
        w = bw.native_workload_declared(c.fixture, c, c.name)
        p, e, q = evgen.to_device(torch_cuda, w.parent, w.events, w.queries)
        variants = [dict(), dict(blocks=3)] + ([dict(chain=True), dict(chain=True, blocks=5),
                                                dict(chain=True, path="chain"),
                                                dict(chain=True, path="chain", blocks=4),
                                                dict(chain=True, path="chain", blocks=3, wide=True)]
                                               if w.chain else [])
        for kw in variants:
            ans = bw.replay(p, w.n_keys, e, q, **kw).cpu().numpy()
            assert bw.sha256_hex(ans.tobytes()) == rec["answers_sha256"], (c.name, kw)
            n += 1
    assert n >= 2 * CHUNK or chunk[1] + CHUNK > len(RUNS[chunk[0]])


@pytest.mark.gpu
@pytest.mark.parametrize("chunk", CHUNKS, ids=chunk_id)
def test_gpu_fuzz_v7_dropin(bw, torch_cuda, chunk):
    for rec, c in cases_of(chunk):
        if c.topology != 0:
            continue
        for blocks in (1, 5):
            plan = bw.v7_plan_declared(c.fixture, c, blocks)
            ans, _, _ = bw.run_v7_plan(plan)
            assert bw.sha256_hex(ans.tobytes()) == rec["answers_sha256"], (c.name, blocks)
