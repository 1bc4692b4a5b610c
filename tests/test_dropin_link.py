"""The reference's own GPU workers link this library unchanged.

oracle/ref.mk (target "dropin") compiles the reference's panel_batch_gpu.cpp (gpu_v7.h),
panel_batch_gpu2.cpp and panel_batch_gpu3.cpp (gpu_v7b.h) and panel_gpu_session.cpp
(gpu_session.h) where their sources lie, with those three headers replaced by
stand-ins that include include/bw_gpu.h, and links them against libbwgpu.so instead
of the reference's kernels.  These CPU tests check that every worker builds, binds
libbwgpu.so, and runs its argument handling and its whole CPU setup up to the first
CUDA call (exit 5 without a GPU, as the reference's CUDA_CHECK returns).  Skipped
where the reference checkout is absent."""
from __future__ import annotations

import os
import subprocess
import zlib
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
WORKERS = ["panel_batch_gpu", "panel_batch_gpu2", "panel_batch_gpu3", "panel_gpu_session"]


@pytest.fixture(scope="module")
def dropin(bw, oracle_mod):
    ref = oracle_mod.reference_dir()
    if ref is None:
        pytest.skip("reference checkout not present")
    bw.build()
    subprocess.run(["make", "-s", "-f", "oracle/ref.mk", f"REF={ref}", "STATES=2049", "dropin"], cwd=ROOT,
                   check=True, capture_output=True)
    return {w: ROOT / "oracle" / "_ref" / f"{w}_2049" for w in WORKERS}


@pytest.mark.parametrize("name", WORKERS)
def test_reference_worker_links_libbwgpu(dropin, name):
    exe = dropin[name]
    assert exe.exists()
    libs = subprocess.run(["ldd", str(exe)], capture_output=True, text=True).stdout
    assert "libbwgpu.so" in libs
    syms = subprocess.run(["nm", "-u", str(exe)], capture_output=True, text=True).stdout
    wanted = {"panel_batch_gpu": "gpu_v7_launch", "panel_batch_gpu2": "gpu_v7b_launch",
              "panel_batch_gpu3": "gpu_v7b_snap_launch", "panel_gpu_session": "gpu_sess_run_launch"}[name]
    assert wanted in syms   # resolved from libbwgpu.so, not defined in the worker
    assert subprocess.run([str(exe), "--bogus"], capture_output=True).returncode == 2


@pytest.mark.parametrize("name", WORKERS)
def test_reference_worker_runs_setup_then_stops_at_cuda(dropin, name, tmp_path):
    if os.environ.get("CUDA_VISIBLE_DEVICES", None) != "" and _has_gpu():
        pytest.skip("a GPU is present: the worker would run to completion")
    fx = tmp_path / "check.bin"
    fx.write_bytes(zlib.decompress((ROOT / "tests" / "golden" / "check.bin.z").read_bytes()))
    r = subprocess.run([str(dropin[name]), "--fixture", str(fx), "--base-id", "check", "--topology", "0", "--seed",
                        "7", "--factor-period", "37", "--q", "2", "--repeat", "0", "--answers",
                        str(tmp_path / "a.bin"), "--json", str(tmp_path / "a.json")],
                       capture_output=True, text=True, env=dict(os.environ, BWH_RANGE_SCOPE="per_state", BWH_BATCH_FORCE="1"))
    assert r.returncode == 5, r.stderr


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
