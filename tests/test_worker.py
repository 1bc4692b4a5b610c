"""The worker binary (bw_worker) keeps the reference GPU worker's process contract
(panel_batch_gpu.cpp:41-299): its CLI, exit codes 2/3/4/5, the raw answer file, the
JSON record written through <json>.tmp and a rename, with answers_sha256,
answers_fn, phases_ns and a "gpu" object.  CPU tests check argument and fixture
errors (they happen before any CUDA call); GPU tests run golden reference cases
through both arms and compare the recorded SHA-256 with the golden values."""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import zlib
from pathlib import Path

import pytest

GOLD = Path(__file__).resolve().parent / "golden"
GOLDEN = json.loads((GOLD / "golden.json").read_text())


def worker(bw) -> Path:
    bw.build()
    return bw._build.WORKER


def fixture_file(tmp_path, name="check") -> Path:
    p = tmp_path / f"{name}.bin"
    p.write_bytes(zlib.decompress((GOLD / f"{name}.bin.z").read_bytes()))
    return p


def run(bw, tmp_path, *args, scope=None, **kw):
    env = {k: v for k, v in os.environ.items() if k not in ("BWH_RANGE_SCOPE", "BWH_STATES", "BWH_V7_BLOCKS")}
    if scope:
        env["BWH_RANGE_SCOPE"] = scope
    return subprocess.run([str(worker(bw)), *map(str, args)], capture_output=True, text=True, env=env,
                          cwd=tmp_path, **kw)


def test_worker_argument_errors_exit_2(bw, tmp_path):
    assert run(bw, tmp_path, "--bogus").returncode == 2
    assert run(bw, tmp_path, "--fixture", "x").returncode == 2                    # no --answers/--json
    assert run(bw, tmp_path, "--fixture", "x", "--answers", "a", "--json", "j", "--arm", "nope").returncode == 2
    assert run(bw, tmp_path, "--fixture", "x", "--answers", "a", "--json", "j", "--q", "two").returncode == 2
    assert run(bw, tmp_path, "--fixture", "x", "--answers", "a", "--json", "j", "--q", "0").returncode == 2
    assert run(bw, tmp_path, "--fixture", "x", "--answers", "a", "--json").returncode == 2   # missing value


def test_worker_fixture_and_case_errors_exit_3(bw, tmp_path):
    common = ["--answers", tmp_path / "a.bin", "--json", tmp_path / "a.json"]
    assert run(bw, tmp_path, "--fixture", tmp_path / "missing.bin", *common).returncode == 3
    bad = tmp_path / "bad.bin"
    img = bytearray(fixture_file(tmp_path).read_bytes())
    img[0:8] = b"BWBASE99"
    bad.write_bytes(bytes(img))
    assert run(bw, tmp_path, "--fixture", bad, *common).returncode == 3
    truncated = tmp_path / "short.bin"
    truncated.write_bytes(bytes(img[:100]))
    assert run(bw, tmp_path, "--fixture", truncated, *common).returncode == 3
    # the v7 block path takes chains only (batch_engine_v7.hpp:708)
    r = run(bw, tmp_path, "--fixture", fixture_file(tmp_path), "--topology", 1, "--arm", "gpu_v7", *common)
    assert r.returncode == 3 and "chains" in r.stderr
    assert not (tmp_path / "a.json").exists()


def test_worker_event_stream_errors(bw, tmp_path):
    common = ["--answers", tmp_path / "a.bin", "--json", tmp_path / "a.json"]
    fx = fixture_file(tmp_path)
    bad = tmp_path / "bad.bwlev"
    bad.write_bytes(b"BWLEV001" + (3).to_bytes(8, "little") + b"\0" * 10)
    assert run(bw, tmp_path, "--fixture", fx, "--events", bad, *common).returncode == 3
    assert run(bw, tmp_path, "--fixture", fx, "--events", tmp_path / "missing.bwlev", *common).returncode == 3
    assert run(bw, tmp_path, "--fixture", fx, "--events", bad, "--arm", "gpu_v7", *common).returncode == 2
    assert not (tmp_path / "a.json").exists()


# ------------------------------------------------------------------------------ GPU
def _cases():
    return [c for c in GOLDEN["cases"] if c["fixture"] == "check"]


@pytest.mark.gpu
@pytest.mark.parametrize("case", _cases(), ids=lambda c: f"t{c['topology']}-s{c['seed']}-f{c['factor_period']}-q{c['q']}"
                         f"{'' if c['per_state'] else '-shared'}")
def test_worker_reproduces_golden(bw, torch_cuda, tmp_path, case):
    fx = fixture_file(tmp_path)
    want = case.get("published") or case.get("reference") or case["oracle"]
    arms = ["gb300"] + (["gpu_v7"] if case["topology"] == 0 else [])
    for arm in arms:
        ans, js = tmp_path / f"{arm}.bin", tmp_path / f"{arm}.json"
        r = run(bw, tmp_path, "--fixture", fx, "--base-id", "check", "--topology", case["topology"], "--seed",
                case["seed"], "--factor-period", case["factor_period"], "--q", case["q"], "--repeat", 0,
                "--states", case["states"], "--arm", arm, "--answers", ans, "--json", js,
                scope="per_state" if case["per_state"] else None)
        assert r.returncode == 0, r.stderr
        rec = json.loads(js.read_text())
        assert not Path(str(js) + ".tmp").exists()
        assert rec["answers_sha256"] == want
        assert hashlib.sha256(ans.read_bytes()).hexdigest() == want
        assert rec["answers_fn"] == case["fnv1a"]
        assert rec["n_answers"] == case["n_answers"] and rec["arm"] == arm
        assert rec["range_scope"] == ("per_state" if case["per_state"] else "shared")
        assert set(rec["phases_ns"]) == {"load", "setup", "execute", "extract", "cleanup"}
        assert {"device", "blocks", "threads", "shared_bytes", "upload_ns", "kernel_ns", "carry_ns", "combine_ns",
                "download_ns"} <= set(rec["gpu"])
        assert rec["full_ns"] > 0 and rec["peak_rss_kb"] > 0 and rec["answers_per_s"] > 0
        assert "GB300" in rec["gpu"]["device"] or rec["gpu"]["device"]


@pytest.mark.gpu
def test_worker_unwritable_answers_exit_4(bw, torch_cuda, tmp_path):
    fx = fixture_file(tmp_path)
    r = run(bw, tmp_path, "--fixture", fx, "--q", 2, "--answers", tmp_path / "no" / "such" / "dir.bin", "--json",
            tmp_path / "x.json", scope="per_state")
    assert r.returncode == 4
    assert not (tmp_path / "x.json").exists()


STREAMS = json.loads((GOLD / "stream_golden.json").read_text())["cases"]


@pytest.mark.gpu
@pytest.mark.parametrize("case", STREAMS, ids=lambda c: c["file"])
def test_worker_event_stream_reproduces_golden(bw, torch_cuda, tmp_path, case):
    fx = fixture_file(tmp_path)
    ev = tmp_path / "s.bwlev"
    ev.write_bytes(zlib.decompress((GOLD / case["file"]).read_bytes()))
    ans, js = tmp_path / "a.bin", tmp_path / "a.json"
    r = run(bw, tmp_path, "--fixture", fx, "--events", ev, "--answers", ans, "--json", js)
    assert r.returncode == 0, r.stderr
    rec = json.loads(js.read_text())
    assert rec["answers_sha256"] == case["answers_sha256"]
    assert hashlib.sha256(ans.read_bytes()).hexdigest() == case["answers_sha256"]
    assert rec["answers_fn"] == case["fnv1a"] and rec["n_answers"] == case["n_answers"]
