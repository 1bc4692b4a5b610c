"""Chain setup on the device: the compact form (bw_native_build_compact) and the
factor expansion (bw_native_expand) against the host event builder.

The compact form keeps the verbatim events (base rows, row edits) with their output
positions and, per group, the timeline of mass updates and factor expansions.  The
CPU tests check that the positions tile the event list and replay the expansion in
numpy: the result must be the host builder's event list once the expansion's
zero-delta events are dropped.  The GPU tests expand on the device, compare with the
same list and replay the chain to the golden answer SHA-256."""
from __future__ import annotations

import json
import zlib
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"
GOLDEN = json.loads((GOLD / "golden.json").read_text())
CASES = [c for c in GOLDEN["cases"] if c["topology"] == 0 and c["fixture"] in ("check", "real3_100k")]


def fixture(name):
    return zlib.decompress((GOLD / f"{name}.bin.z").read_bytes())


def case_id(c):
    return f"{c['fixture']}-s{c['seed']}-f{c['factor_period']}-q{c['q']}{'' if c['per_state'] else '-shared'}"


def expected(c):
    return c.get("published") or c.get("reference") or c["oracle"]


def emulate(cp):
    """numpy replay of bw_native_expand's semantics."""
    ev = np.zeros(cp["n_events"], dtype=[("state", "<u4"), ("key", "<u4"), ("delta", "<i8")])
    ev[cp["fixed_pos"]] = cp["fixed"]
    with np.errstate(over="ignore"):
        for g in range(cp["n_groups"]):
            s0, s1 = cp["sup_off"][g], cp["sup_off"][g + 1]
            cls = cp["sup_cls"][s0:s1]
            mass = cp["base_mass"][s0:s1].astype(np.uint64)
            for r in cp["tl"][cp["tl_off"][g]:cp["tl_off"][g + 1]]:
                if r["idx"] >= 0:
                    mass[r["idx"]] += np.uint64(int(r["value"]) & 0xFFFFFFFFFFFFFFFF)
                else:
                    o = int(r["out"])
                    ev["state"][o:o + len(cls)] = r["state"]
                    ev["key"][o:o + len(cls)] = cls
                    ev["delta"][o:o + len(cls)] = (mass * np.uint64(int(r["value"]) & 0xFFFFFFFFFFFFFFFF)).view(np.int64)
    return ev


def nonzero(ev):
    return ev[ev["delta"] != 0]


@pytest.mark.parametrize("case", CASES, ids=case_id)
def test_compact_form_tiles_and_expands_to_host_events(bw, case):
    fx = fixture(case["fixture"])
    cp = bw.native_compact(fx, case["states"], case["seed"], case["factor_period"], case["q"], case["per_state"])
    host = bw.native_workload(fx, case["states"], 0, case["seed"], case["factor_period"], case["q"],
                              case["per_state"])
    # positions: the verbatim events and the expansion ranges partition [0, n_events)
    cover = np.zeros(cp["n_events"], dtype=np.int32)
    np.add.at(cover, cp["fixed_pos"], 1)
    exp = cp["tl"][cp["tl"]["idx"] < 0]
    for g in range(cp["n_groups"]):
        n = cp["sup_off"][g + 1] - cp["sup_off"][g]
        for r in cp["tl"][cp["tl_off"][g]:cp["tl_off"][g + 1]]:
            if r["idx"] < 0:
                cover[r["out"]:r["out"] + n] += 1
            else:
                assert 0 <= r["idx"] < n
        st = cp["tl"][cp["tl_off"][g]:cp["tl_off"][g + 1]]["state"]
        assert np.all(np.diff(st) >= 0)
    assert np.all(cover == 1) and len(exp) > 0
    ev = emulate(cp)
    assert np.all(np.diff(ev["state"].astype(np.int64)) >= 0)
    np.testing.assert_array_equal(nonzero(ev), nonzero(host.events))
    np.testing.assert_array_equal(cp["queries"], host.queries)
    assert cp["n_keys"] == host.n_keys


def test_compact_form_takes_chains_only(bw):
    import ctypes as C

    def run(L, fx):
        L.bw_native_build_compact.argtypes = [C.c_void_p, C.POINTER(bw.BwNativeSpec), C.c_void_p]
        out = C.c_void_p()
        return L.bw_native_build_compact(fx, C.byref(bw.BwNativeSpec(2049, 1, 7, 4, 2, 1, -1)), C.byref(out))
    assert bw._with_fixture(fixture("check"), run) == 2   # bushy tree: the host builder's job


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=case_id)
def test_gpu_expansion_matches_host_and_golden(bw, torch_cuda, case):
    import torch
    fx = fixture(case["fixture"])
    cp = bw.native_compact(fx, case["states"], case["seed"], case["factor_period"], case["q"], case["per_state"])
    ev = bw.expand_events(cp)
    got = ev.cpu().numpy().view([("state", "<u4"), ("key", "<u4"), ("delta", "<i8")]).reshape(-1)
    np.testing.assert_array_equal(got, emulate(cp))
    dev = ev.device
    p = torch.from_numpy(cp["parent"]).to(dev)
    q = torch.from_numpy(cp["queries"].view(np.int32).reshape(-1, 3)).to(dev)
    for kw in (dict(chain=True), dict(chain=True, path="chain", wide=True), dict(chain=True, path="general")):
        ans = bw.replay(p, cp["n_keys"], ev, q, **kw).cpu().numpy()
        assert bw.sha256_hex(ans.tobytes()) == expected(case), kw
