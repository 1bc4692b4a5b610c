"""CPU tests of the oracle (test infrastructure) against the reference's golden
vectors and against itself across independent algorithms."""
from __future__ import annotations

import hashlib
import json
import zlib
from pathlib import Path

import numpy as np
import pytest

import evgen

GOLD = Path(__file__).resolve().parent / "golden"
GOLDEN = json.loads((GOLD / "golden.json").read_text())


def fixture(name: str) -> bytes:
    return zlib.decompress((GOLD / f"{name}.bin.z").read_bytes())


def test_sha256_known_answers(oracle_mod):
    # FIPS 180-4 examples and lengths around the padding boundaries
    assert oracle_mod.sha256_hex(b"abc") == \
        "ba7816bf8f01cfea414140de5dae2223b00361a396177a9cb410ff61f20015ad"
    assert oracle_mod.sha256_hex(b"") == \
        "e3b0c44298fc1c149afbf4c8996fb92427ae41e4649b934ca495991b7852b855"
    data = bytes(range(256)) * 3
    for n in (1, 55, 56, 57, 63, 64, 65, 119, 120, 128, 700):
        assert oracle_mod.sha256_hex(data[:n]) == hashlib.sha256(data[:n]).hexdigest()


def test_fnv1a(oracle_mod):
    # common.hpp:396-400 seeds FNV-1a with 1469598103934665603 (not the usual
    # 14695981039346656037); the published answers_fn values depend on it.
    def ref(b):
        h = 1469598103934665603
        for x in b:
            h = ((h ^ x) * 1099511628211) % (1 << 64)
        return h
    assert oracle_mod.fnv1a(b"") == 1469598103934665603
    for b in (b"a", bytes(range(200))):
        assert oracle_mod.fnv1a(b) == ref(b)
    # the reference's own JSON record for the 1d_q2 golden case
    # (results/general_router_final2_20261102/raw/1d_q2_batch_v7fix_r0.json)
    case = next(c for c in GOLDEN["cases"] if c["seed"] == 20261291)
    assert case["fnv1a"] == "24552c03820e7040"


def test_golden_fixture_bytes():
    for name, sha in GOLDEN["fixtures"].items():
        assert hashlib.sha256(fixture(name)).hexdigest() == sha


def test_fixture_generator_reproduces_reference_tool():
    import sys
    sys.path.insert(0, str(GOLD))
    import make_golden
    img = make_golden.make_fixture(2000, 4, 20261131, 86_400_000_000)
    assert hashlib.sha256(img).hexdigest() == GOLDEN["fixtures"]["check"]


def test_fixture_rejects_malformed(oracle_mod):
    img = bytearray(fixture("check"))
    with pytest.raises(ValueError):
        oracle_mod.Fixture(b"BWBASE01" + bytes(img[8:]))
    with pytest.raises(ValueError):
        oracle_mod.Fixture(bytes(img[:100]))
    bad = bytearray(img)
    bad[64 + 2000 * 24: 64 + 2000 * 24 + 8] = (0).to_bytes(8, "little")  # factor 0
    with pytest.raises(ValueError):
        oracle_mod.Fixture(bytes(bad))


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=lambda c: f"{c['fixture']}-t{c['topology']}-s{c['seed']}-f{c['factor_period']}-q{c['q']}")
def test_direct_scan_matches_golden(oracle_mod, case):
    fx = oracle_mod.Fixture(fixture(case["fixture"]))
    ans = oracle_mod.direct_scan(fx, case["states"], case["topology"], case["seed"],
                                 case["factor_period"], case["q"], case["per_state"])
    sha = oracle_mod.sha256_hex(ans.tobytes())
    assert sha == case["oracle"]
    for k in ("published", "reference"):
        if k in case:
            assert sha == case[k]


@pytest.mark.parametrize("kind", ["chain", "bushy", "star", "fork"])
def test_event_checkers_agree(oracle_mod, kind):
    rng = np.random.default_rng(11)
    S, C = 300, 97
    parent = evgen.make_tree(S, kind, rng)
    ev = evgen.make_events(S, C, 4000, rng, zipf=1.1)
    qs = evgen.make_queries(S, C, 3000, rng)
    a = oracle_mod.ev_bruteforce(parent, ev, qs)
    b = oracle_mod.ev_sweep(parent, C, ev, qs)
    np.testing.assert_array_equal(a, b)
    if kind == "chain":
        for blocks in (1, 3, 16):
            np.testing.assert_array_equal(a, oracle_mod.ev_blocks(parent, C, ev, qs, blocks=blocks))


def test_event_checkers_wrap_int64(oracle_mod):
    rng = np.random.default_rng(5)
    S, C = 64, 33
    parent = evgen.make_tree(S, "fork", rng)
    ev = evgen.make_events(S, C, 2000, rng, big=True)
    qs = evgen.make_queries(S, C, 500, rng)
    np.testing.assert_array_equal(oracle_mod.ev_bruteforce(parent, ev, qs),
                                  oracle_mod.ev_sweep(parent, C, ev, qs))


def test_event_sweep_prefix_sample(oracle_mod):
    rng = np.random.default_rng(3)
    S, C = 200, 50
    parent = evgen.make_tree(S, "fork", rng)
    ev = evgen.make_events(S, C, 3000, rng)
    qs = evgen.make_queries(S, C, 800, rng)
    full = oracle_mod.ev_sweep(parent, C, ev, qs)
    part, done, secs = oracle_mod.ev_sweep_prefix(parent, C, ev, qs, 50)
    assert 0 < done < len(qs) and secs >= 0
    answered = part != 0
    np.testing.assert_array_equal(part[answered], full[answered])


def test_event_inputs_rejected(oracle_mod):
    rng = np.random.default_rng(1)
    parent = evgen.make_tree(10, "chain", rng)
    ev = evgen.make_events(10, 8, 20, rng)
    qs = evgen.make_queries(10, 8, 5, rng)
    bad = ev.copy()
    bad["key"][0] = 8
    with pytest.raises(ValueError):
        oracle_mod.ev_sweep(parent, 8, bad, qs)
    badp = parent.copy()
    badp[5] = 7
    with pytest.raises(ValueError):
        oracle_mod.ev_sweep(badp, 8, ev, qs)


def test_forest_oracle_is_per_tree_replay(oracle_mod):
    """ev_forest answers each tree's queries from that tree alone (checked against
    the ancestor-walk brute force)."""
    rng = np.random.default_rng(3)
    soff, eoff, qoff, keys, parts = [0], [0], [0], [], ([], [], [])
    for t in range(6):
        S, C = int(rng.integers(1, 300)), int(rng.integers(1, 500))
        par = evgen.make_tree(S, ["chain", "fork", "star"][t % 3], rng) if S > 1 else np.array([-1], np.int32)
        ev = evgen.make_events(S, C, int(rng.integers(0, 3000)), rng)
        qs = evgen.make_queries(S, C, int(rng.integers(0, 400)), rng)
        for lst, x in zip(parts, (par, ev, qs)):
            lst.append(x)
        soff.append(soff[-1] + S); eoff.append(eoff[-1] + len(ev)); qoff.append(qoff[-1] + len(qs)); keys.append(C)
    F = (np.array(soff), np.array(eoff), np.array(qoff), np.array(keys), np.concatenate(parts[0]),
         np.concatenate(parts[1]), np.concatenate(parts[2]))
    brute = oracle_mod.ev_forest(*F, fn=lambda p, C, e, q: oracle_mod.ev_bruteforce(p, e, q))
    np.testing.assert_array_equal(oracle_mod.ev_forest(*F), brute)
