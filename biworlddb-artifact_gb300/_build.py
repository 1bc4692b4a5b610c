"""In-tree build of the native libraries (no cmake, no pip install).

* ``libbwgpu.so``  -- the CUDA kernels and the C ABI of include/bw_gpu.h, compiled
  for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``);
* ``libbwhost.so`` -- host C++: BWBASE02 fixtures, the declared workload and the
  reference-native event builder, synthetic workload generators, SHA-256
  (include/bw_host.h);
* ``bw_worker``    -- the worker binary with the reference's CLI/JSON contract.

Translation units compile in parallel; a rebuild only happens when a source is
newer than its output.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"

GPU_LIB = PKG / "libbwgpu.so"
HOST_LIB = PKG / "libbwhost.so"
WORKER = PKG / "bw_worker"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found: the GB300 kernels cannot be built")


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _gpu_sources():
    return sorted(CSRC.glob("*.cu"))


def _host_sources():
    return sorted(p for p in CSRC.glob("*.cpp") if p.name != "worker_main.cpp")


def _deps():
    return (list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.cpp"))
            + list(CSRC.glob("*.hpp")) + list(INCLUDE.glob("*.h")))


def build(force: bool = False, verbose: bool = False) -> None:
    deps = _deps()
    jobs = []
    objdir = PKG / "_build"
    objdir.mkdir(exist_ok=True)
    nvcc = _nvcc()
    gpu_objs = []
    if force or _stale(GPU_LIB, deps):
        for src in _gpu_sources():
            obj = objdir / (src.stem + ".o")
            gpu_objs.append(obj)
            jobs.append([nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                         "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(src), "-o", str(obj)])
    host_objs = []
    if force or _stale(HOST_LIB, deps) or _stale(WORKER, deps):
        for src in _host_sources():
            obj = objdir / (src.stem + ".host.o")
            host_objs.append(obj)
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off",
                         "-Wall", "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(src), "-o", str(obj)])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for j in jobs]
    errors = []
    for j, p in procs:
        out, _ = p.communicate()
        if p.returncode:
            errors.append(f"{' '.join(j)}\n{out}")
        elif verbose and out:
            print(out)
    if errors:
        raise RuntimeError("native build failed:\n" + "\n".join(errors))
    if gpu_objs:
        subprocess.run([nvcc, *ARCH, "-shared", "-o", str(GPU_LIB), *map(str, gpu_objs)], check=True)
    if host_objs:
        subprocess.run(["g++", "-shared", "-fopenmp", "-o", str(HOST_LIB), *map(str, host_objs), "-ldl"],
                       check=True)
        # the worker: host objects linked in, the CUDA library by rpath
        subprocess.run([nvcc, *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fopenmp,-ffp-contract=off",
                        "-I", str(INCLUDE), "-I", str(CSRC), str(CSRC / "worker_main.cpp"), *map(str, host_objs),
                        "-L", str(PKG), "-lbwgpu", "-lgomp", "-ldl", f"-Xlinker=-rpath,{PKG}", "-o", str(WORKER)],
                       check=True)
