"""BWLEV001 event-stream ingest (bw_stream_build) against the reference.

The golden streams are the reference's own emitter output (emit_events.cpp,
tests/golden/make_stream_golden.py) for reference-native cases of the ``check``
fixture whose answer SHA-256 the golden set already pins.  The oracle replays a
stream the way the reference's stream consumers do (external/dd_probe/src/main.rs)
and must reproduce that SHA; the front end compiles the stream into a linear-chain
event workload, which the oracle's event sweep (CPU) and the CUDA replay (GPU,
chain and general paths) must answer with the same bits."""
from __future__ import annotations

import hashlib
import json
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"
SG = json.loads((GOLD / "stream_golden.json").read_text())
FIXTURE = zlib.decompress((GOLD / "check.bin.z").read_bytes())


def stream(case) -> bytes:
    return zlib.decompress((GOLD / case["file"]).read_bytes())


def case_id(c):
    return f"t{c['topology']}-s{c['seed']}-f{c['factor_period']}-q{c['q']}"


@pytest.mark.parametrize("case", SG["cases"], ids=case_id)
def test_stream_oracle_matches_reference(oracle_mod, case):
    data = stream(case)
    assert hashlib.sha256(data).hexdigest() == case["stream_sha256"]
    ans = oracle_mod.stream_answers(FIXTURE, data)
    assert ans.size == case["n_answers"]
    assert oracle_mod.sha256_hex(ans.tobytes()) == case["answers_sha256"]


@pytest.mark.parametrize("case", SG["cases"], ids=case_id)
def test_stream_front_end_matches_reference(bw, oracle_mod, case):
    w, slot, n_answers = bw.stream_workload(FIXTURE, stream(case))
    assert n_answers == case["n_answers"] and w.chain
    assert np.all(np.diff(w.events["state"].astype(np.int64)) >= 0)
    assert np.all(np.diff(w.queries["state"].astype(np.int64)) >= 0)
    got = oracle_mod.ev_sweep(w.parent, w.n_keys, w.events, w.queries)
    ans = bw.scatter_answers(got, slot, n_answers)
    assert bw.sha256_hex(ans.tobytes()) == case["answers_sha256"]
    assert f"{bw.fnv1a(ans.tobytes()):016x}" == case["fnv1a"]


def test_stream_rejects_malformed(bw):
    data = bytearray(stream(SG["cases"][0]))
    n = struct.unpack_from("<Q", data, 8)[0]

    def rejected(img):
        with pytest.raises(ValueError):
            bw.stream_workload(FIXTURE, bytes(img))

    bad = bytearray(data)
    bad[0:8] = b"BWLEV002"
    rejected(bad)
    rejected(data[:-1])                        # truncated record
    bad = bytearray(data)
    struct.pack_into("<Q", bad, 8, n + 1)      # count past the end
    rejected(bad)
    rec = 16 + 36 * 5
    bad = bytearray(data)
    struct.pack_into("<I", bad, rec, 7)        # unknown kind
    rejected(bad)
    first_row = next(i for i in range(n) if struct.unpack_from("<I", data, 16 + 36 * i)[0] == 0)
    bad = bytearray(data)
    struct.pack_into("<i", bad, 16 + 36 * first_row + 12, 99)   # group outside the fixture
    rejected(bad)
    bad = bytearray(data)
    struct.pack_into("<i", bad, 16 + 36 * first_row + 16, 2)    # weight other than +-1
    rejected(bad)
    qs = [i for i in range(n) if struct.unpack_from("<I", data, 16 + 36 * i)[0] == 2
          and struct.unpack_from("<I", data, 16 + 36 * i + 4)[0] > 0]
    bad = bytearray(data)
    bad[16 + 36 * qs[1]:16 + 36 * qs[1] + 36] = data[16 + 36 * qs[0]:16 + 36 * qs[0] + 36]   # (state, k) twice
    rejected(bad)
    # an empty stream: the base rows only, no answers
    w, slot, n_answers = bw.stream_workload(FIXTURE, b"BWLEV001" + struct.pack("<Q", 0))
    assert n_answers == 0 and len(w.queries) == 0 and len(w.events) > 0


def test_wide_delta_rule(bw):
    """The int64-window hint: more than one delta in 64 outside (-2^19, 2^19)."""
    ev = np.zeros(640, dtype=[("state", "<u4"), ("key", "<u4"), ("delta", "<i8")])
    assert not bw.wide_deltas(ev)
    ev["delta"][:10] = 1 << 19          # 10 of 640: one in 64, not more
    assert not bw.wide_deltas(ev)
    ev["delta"][:11] = 1 << 19
    assert bw.wide_deltas(ev)
    ev["delta"][:11] = (1 << 19) - 1
    assert not bw.wide_deltas(ev)
    ev["delta"][:11] = -(1 << 19)
    assert bw.wide_deltas(ev)


@pytest.mark.gpu
@pytest.mark.parametrize("case", SG["cases"], ids=case_id)
def test_gpu_stream_replay(bw, torch_cuda, case):
    import evgen
    w, slot, n_answers = bw.stream_workload(FIXTURE, stream(case))
    p, e, q = evgen.to_device(torch_cuda, w.parent, w.events, w.queries)
    assert bw.wide_deltas(w.events)   # amount x factor products: the int64 window's case
    for kw in (dict(chain=True), dict(chain=True, path="chain"), dict(chain=True, path="chain", blocks=7),
               dict(chain=True, path="chain", wide=True), dict(chain=True, path="chain", blocks=5, wide=True),
               dict(chain=True, path="general"), dict()):
        got = bw.replay(p, w.n_keys, e, q, **kw).cpu().numpy()
        ans = bw.scatter_answers(got, slot, n_answers)
        assert bw.sha256_hex(ans.tobytes()) == case["answers_sha256"], kw
