"""Reference-native parity: BWBASE02 fixtures + declared workloads compiled by the
host front end (libbwhost.so) must reproduce the reference's answer hashes.

CPU tests check the host front end through the oracle's event-model replay and the
v7 plan through a Python port of the reference's block executor; GPU tests run the
same cases through the CUDA replay and through the gpu_v7.h drop-in entry points."""
from __future__ import annotations

import json
import zlib
from pathlib import Path

import numpy as np
import pytest

import v7_emul

GOLD = Path(__file__).resolve().parent / "golden"
GOLDEN = json.loads((GOLD / "golden.json").read_text())
CASES = GOLDEN["cases"]
LARGE = GOLDEN["large_cases"]


def fixture(name: str) -> bytes:
    return zlib.decompress((GOLD / f"{name}.bin.z").read_bytes())


def cid(c):
    scope = "" if c.get("per_state", True) else "-shared"
    return f"{c['fixture']}-S{c['states']}-t{c['topology']}-s{c['seed']}-f{c['factor_period']}-q{c['q']}{scope}"


def expected(c):
    return c.get("published") or c.get("reference") or c["oracle"]


@pytest.mark.parametrize("case", CASES, ids=cid)
def test_front_end_events_reproduce_golden(bw, oracle_mod, case):
    w = bw.native_workload(fixture(case["fixture"]), case["states"], case["topology"], case["seed"],
                           case["factor_period"], case["q"], case["per_state"])
    assert len(w.queries) == case["n_answers"]
    ans = oracle_mod.ev_sweep(w.parent, w.n_keys, w.events, w.queries)
    assert bw.sha256_hex(ans.tobytes()) == expected(case)
    assert f"{bw.fnv1a(ans.tobytes()):016x}" == case["fnv1a"]


@pytest.mark.parametrize("case", [c for c in CASES if c["topology"] == 0 and c["q"] == 2], ids=cid)
def test_v7_plan_reproduces_golden(bw, case):
    plan = bw.v7_plan(fixture(case["fixture"]), case["states"], case["seed"], case["factor_period"],
                      case["q"], blocks=7, per_state=case["per_state"])
    ans, _, _ = v7_emul.run(plan)
    assert bw.sha256_hex(ans.tobytes()) == expected(case)


def test_host_sha_matches_oracle(bw, oracle_mod):
    data = np.arange(1000, dtype=np.int64).tobytes()
    for n in (0, 3, 55, 64, 100, 8000):
        assert bw.sha256_hex(data[:n]) == oracle_mod.sha256_hex(data[:n])
        assert bw.fnv1a(data[:n]) == oracle_mod.fnv1a(data[:n])


@pytest.mark.parametrize("topology,factor_pct", [(0, 30), (1, 10), (2, 0), (0, 100)])
def test_counter_based_edits_match_sequential_oracle(bw, oracle_mod, topology, factor_pct):
    """The declared edit stream drawn in two phases (sequential op pass, parallel
    materialisation from the counter property) equals the sequential draw order of
    the oracle's make_workload restatement, on the BWH_FACTOR_PCT path too."""
    fx = fixture("check")
    w = bw.native_workload(fx, 257, topology, 13, 4, 2, True, factor_pct)
    want = oracle_mod.direct_scan(oracle_mod.Fixture(fx), 257, topology, 13, 4, 2, True, factor_pct)
    got = oracle_mod.ev_sweep(w.parent, w.n_keys, w.events, w.queries)
    np.testing.assert_array_equal(got, want)


def test_streaming_digest_equals_one_shot(bw):
    """The extract digests chunk by chunk: any split gives the one-shot SHA-256/FNV-1a."""
    rng = np.random.default_rng(5)
    data = rng.integers(0, 256, 300_001, dtype=np.uint8).tobytes()
    for cuts in ([], [1], [63, 64, 65], [55, 56, 57, 120], list(rng.integers(0, len(data), 40))):
        d = bw.Digest()
        prev = 0
        for c in sorted(cuts) + [len(data)]:
            d.update(data[prev:c])
            prev = c
        sha, fnv = d.final()
        assert sha == bw.sha256_hex(data) and fnv == bw.fnv1a(data)
    assert bw.Digest().final()[0] == bw.sha256_hex(b"")


def test_platform_and_portable_sha_agree(bw, tmp_path):
    """The digest uses the platform SHA-256 (OpenSSL EVP, found at run time) unless
    BW_SHA=sw selects the portable FIPS 180-4 code: both give hashlib's digest."""
    import hashlib
    import os
    import subprocess
    import sys
    data = np.random.default_rng(9).integers(0, 256, 1_000_003, dtype=np.uint8).tobytes()
    (tmp_path / "d.bin").write_bytes(data)
    code = ("import importlib, sys; sys.path.insert(0, sys.argv[1]); "
            "bw = importlib.import_module('biworlddb-artifact_gb300'); "
            "d = bw.Digest(); b = open(sys.argv[2], 'rb').read(); d.update(b[:777]); d.update(b[777:]); "
            "print(bw.sha256_hex(b), d.final()[0])")
    root = str(Path(__file__).resolve().parent.parent)
    for mode in ("sw", "hw"):
        env = dict(os.environ, BW_SHA=mode)
        out = subprocess.run([sys.executable, "-c", code, root, str(tmp_path / "d.bin")], env=env,
                             capture_output=True, text=True, check=True).stdout.split()
        assert out == [hashlib.sha256(data).hexdigest()] * 2, mode


def test_front_end_rejects_bad_fixture(bw):
    img = bytearray(fixture("check"))
    img[0:8] = b"BWBASE99"
    with pytest.raises(ValueError):
        bw.native_workload(bytes(img), 33, 0, 1, 4, 2)


# ------------------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=cid)
def test_gpu_replay_reproduces_golden(bw, torch_cuda, case):
    import evgen
    w = bw.native_workload(fixture(case["fixture"]), case["states"], case["topology"], case["seed"],
                           case["factor_period"], case["q"], case["per_state"])
    p, e, q = evgen.to_device(torch_cuda, w.parent, w.events, w.queries)
    ans = bw.replay(p, w.n_keys, e, q, chain=w.chain).cpu().numpy()
    assert bw.sha256_hex(ans.tobytes()) == expected(case)
    if w.chain and w.n_keys <= 32768:   # the single-pass chain path, forced on this query-heavy case
        for blocks in (0, 6):
            ans = bw.replay(p, w.n_keys, e, q, chain=True, path="chain", blocks=blocks).cpu().numpy()
            assert bw.sha256_hex(ans.tobytes()) == expected(case)


@pytest.mark.gpu
@pytest.mark.parametrize("case", LARGE, ids=cid)
def test_gpu_replay_large_reference_case(bw, torch_cuda, case):
    import evgen
    w = bw.native_workload(fixture(case["fixture"]), case["states"], case["topology"], case["seed"],
                           case["factor_period"], case["q"], case["per_state"])
    p, e, q = evgen.to_device(torch_cuda, w.parent, w.events, w.queries)
    for chain in (True, False):
        ans = bw.replay(p, w.n_keys, e, q, chain=chain).cpu().numpy()
        assert bw.sha256_hex(ans.tobytes()) == case["reference"]


@pytest.mark.gpu
@pytest.mark.parametrize("case", [c for c in CASES if c["topology"] == 0], ids=cid)
@pytest.mark.parametrize("blocks", [1, 9, 64])
def test_gpu_v7_dropin_reproduces_golden(bw, torch_cuda, case, blocks):
    plan = bw.v7_plan(fixture(case["fixture"]), case["states"], case["seed"], case["factor_period"],
                      case["q"], blocks=blocks, per_state=case["per_state"])
    ans, dV, lvals = bw.run_v7_plan(plan)
    assert bw.sha256_hex(ans.tobytes()) == expected(case)
    if case["q"] in (2, 8) and blocks == 9:
        # intermediate outputs of gpu_v7_launch equal the reference block executor's
        e_ans, e_dV, e_lvals = v7_emul.run(plan)
        np.testing.assert_array_equal(dV.reshape(e_dV.shape), e_dV)
        np.testing.assert_array_equal(lvals, e_lvals)


@pytest.mark.gpu
@pytest.mark.parametrize("case", LARGE, ids=cid)
def test_gpu_v7_dropin_large_reference_case(bw, torch_cuda, case):
    plan = bw.v7_plan(fixture(case["fixture"]), case["states"], case["seed"], case["factor_period"],
                      case["q"], blocks=128)
    ans, _, _ = bw.run_v7_plan(plan)
    assert bw.sha256_hex(ans.tobytes()) == case["reference"]


@pytest.mark.gpu
@pytest.mark.parametrize("case", [c for c in CASES if c["topology"] == 0], ids=cid)
@pytest.mark.parametrize("blocks", [1, 9, 64])
def test_gpu_v7b_and_session_reproduce_golden(bw, torch_cuda, case, blocks):
    """The compact (gpu_v7b.h) and session (gpu_session.h) drop-in entries: device
    snapshots equal the host plan's block-start deviations, and the answers hash to
    the golden value (session: two query batches from the same snapshots)."""
    plan = bw.v7_plan(fixture(case["fixture"]), case["states"], case["seed"], case["factor_period"],
                      case["q"], blocks=blocks, per_state=case["per_state"])
    ans, snap = bw.run_v7b_plan(plan)
    np.testing.assert_array_equal(snap[:plan["devbuf"].size], plan["devbuf"])
    assert bw.sha256_hex(ans.tobytes()) == expected(case)
    ans, snap = bw.run_v7b_plan(plan, session=True, batches=2)
    np.testing.assert_array_equal(snap[:plan["devbuf"].size], plan["devbuf"])
    assert bw.sha256_hex(ans.tobytes()) == expected(case)


@pytest.mark.gpu
@pytest.mark.parametrize("case", LARGE, ids=cid)
def test_gpu_session_large_reference_case(bw, torch_cuda, case):
    plan = bw.v7_plan(fixture(case["fixture"]), case["states"], case["seed"], case["factor_period"],
                      case["q"], blocks=128)
    ans, _ = bw.run_v7b_plan(plan, session=True)
    assert bw.sha256_hex(ans.tobytes()) == case["reference"]
