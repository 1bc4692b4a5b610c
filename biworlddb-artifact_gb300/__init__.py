"""GB300-native BiWorldDB version-tree range-sum executor (host-side mirror).

The compute path is the CUDA library ``libbwgpu.so`` (include/bw_gpu.h), driven
here through ctypes with PyTorch supplying device memory and streams.  There is
no CPU fallback: every entry point raises if the CUDA library or a GPU is
missing.

Event-model operator (the reference's per-state answer over endpoint classes,
oracle.cpp:357-422 / batch_engine_v7.hpp:832-968):

    answers = replay(parent, n_keys, events, queries)

* ``parent``: int32[S] (parent[0] = -1, parent[v] < v), the version tree;
* ``events``: int64[E, 2] rows ``(state | key << 32, delta)`` -- the 16-byte
  ``BwEvent`` record -- grouped by state;
* ``queries``: int32[Q, 3] rows ``(state, lo, hi)`` -- the 12-byte ``BwQuery``
  record -- grouped by state;
* returns int64[Q]: for query j the wrapping int64 sum of the deltas of events on
  the root path of its state with key in [lo, hi) (0 when hi <= lo).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import _build, workloads  # noqa: F401

PKG = _build.PKG

BW_EINVAL = 1001
BW_REPLAY_CHAIN_HINT = 1
BW_REPLAY_TIMING = 2
STAGES = ["ingest", "linearise", "blocks", "prepare", "carry", "sweep"]
STATUS_NAMES = {0: "ok", 1: "events not grouped by state", 2: "event key out of range",
                3: "queries not grouped by state", 4: "query bound out of range",
                5: "bad parent array", 6: "too many key slices in a block",
                7: "state id out of range"}


class BwReplayArgs(C.Structure):
    _fields_ = [("n_states", C.c_int32), ("parent", C.c_void_p), ("n_keys", C.c_uint32),
                ("n_events", C.c_int64), ("events", C.c_void_p), ("n_queries", C.c_int64),
                ("queries", C.c_void_p), ("answers", C.c_void_p), ("workspace", C.c_void_p),
                ("workspace_bytes", C.c_size_t), ("stream", C.c_void_p), ("blocks", C.c_int32),
                ("flags", C.c_int32)]


GPU_SYMBOLS = ["gpu_v7_launch", "gpu_combine_launch", "bw_v7_carry_launch",
               "bw_replay_workspace_size", "bw_replay_launch", "bw_replay_status",
               "bw_replay_last_info", "bw_replay_timing_reset", "bw_replay_stage_times",
               "bw_device_info"]

_gpu = None


def build(force: bool = False) -> None:
    """Compile the native libraries in place (nvcc for sm_103a, g++)."""
    _build.build(force=force)


def gpu_lib(build_if_missing: bool = True):
    """The loaded CUDA library; raises if it cannot be built or loaded."""
    global _gpu
    if _gpu is None:
        if build_if_missing:
            _build.build()
        if not _build.GPU_LIB.exists():
            raise RuntimeError(f"CUDA library missing: {_build.GPU_LIB}")
        L = C.CDLL(str(_build.GPU_LIB))
        L.bw_replay_workspace_size.argtypes = [C.POINTER(BwReplayArgs), C.POINTER(C.c_size_t)]
        L.bw_replay_launch.argtypes = [C.POINTER(BwReplayArgs)]
        L.bw_replay_status.argtypes = [C.POINTER(BwReplayArgs), C.POINTER(C.c_int32)]
        L.bw_replay_last_info.argtypes = [C.POINTER(BwReplayArgs), C.POINTER(C.c_int32),
                                          C.POINTER(C.c_int32)]
        L.bw_device_info.argtypes = [C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.bw_replay_stage_times.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_int32)]
        L.bw_v7_carry_launch.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p]
        L.gpu_v7_launch.argtypes = [C.c_void_p]
        L.gpu_combine_launch.argtypes = [C.c_void_p]
        _gpu = L
    return _gpu


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("the GB300 executor needs a CUDA device; no CPU fallback exists")
    return torch


def _check(rc: int, what: str) -> None:
    if rc:
        raise RuntimeError(f"{what} failed with code {rc}")


class Replay:
    """Reusable replay plan: holds the device workspace for one input shape."""

    def __init__(self, parent, n_keys: int, n_events: int, n_queries: int, *, blocks: int = 0,
                 chain: bool = False, timing: bool = False, device=None):
        torch = _torch()
        self.lib = gpu_lib()
        self.device = device or parent.device
        self.args = BwReplayArgs()
        a = self.args
        a.n_states = int(parent.numel())
        a.n_keys = int(n_keys)
        a.n_events = int(n_events)
        a.n_queries = int(n_queries)
        a.blocks = int(blocks)
        a.flags = (BW_REPLAY_CHAIN_HINT if chain else 0) | (BW_REPLAY_TIMING if timing else 0)
        nbytes = C.c_size_t(0)
        _check(self.lib.bw_replay_workspace_size(C.byref(a), C.byref(nbytes)), "workspace size")
        self.workspace = torch.empty(max(int(nbytes.value), 256), dtype=torch.uint8, device=self.device)
        a.workspace = self.workspace.data_ptr()
        a.workspace_bytes = self.workspace.numel()

    def launch(self, parent, events, queries, answers, stream=None) -> None:
        """Enqueue the replay on `stream` (default: torch's current stream)."""
        torch = _torch()
        a = self.args
        if parent.dtype != torch.int32 or events.dtype != torch.int64 or queries.dtype != torch.int32:
            raise TypeError("parent int32, events int64[E,2], queries int32[Q,3] expected")
        if events.numel() != 2 * a.n_events or queries.numel() != 3 * a.n_queries:
            raise ValueError("input sizes differ from the plan")
        for t in (parent, events, queries, answers):
            if not t.is_cuda or not t.is_contiguous():
                raise ValueError("inputs must be contiguous CUDA tensors")
        a.parent = parent.data_ptr()
        a.events = events.data_ptr() if a.n_events else None
        a.queries = queries.data_ptr() if a.n_queries else None
        a.answers = answers.data_ptr() if a.n_queries else None
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        a.stream = s.cuda_stream
        _check(self.lib.bw_replay_launch(C.byref(a)), "bw_replay_launch")

    def status(self) -> int:
        st = C.c_int32(0)
        _check(self.lib.bw_replay_status(C.byref(self.args), C.byref(st)), "bw_replay_status")
        return int(st.value)

    def timing_reset(self) -> None:
        _check(self.lib.bw_replay_timing_reset(), "bw_replay_timing_reset")

    def stage_times(self):
        """(per-stage milliseconds summed over the timed launches since the last
        timing_reset(), number of launches); synchronises."""
        ms = (C.c_float * len(STAGES))()
        n = C.c_int32(0)
        _check(self.lib.bw_replay_stage_times(ms, C.byref(n)), "bw_replay_stage_times")
        return dict(zip(STAGES, [float(x) for x in ms])), int(n.value)

    def info(self):
        k, b = C.c_int32(0), C.c_int32(0)
        self.lib.bw_replay_last_info(C.byref(self.args), C.byref(k), C.byref(b))
        return int(k.value), int(b.value)


def replay(parent, n_keys: int, events, queries, *, blocks: int = 0, chain: bool = False,
           check: bool = True):
    """One replay on the current CUDA stream; returns int64 answers on the device."""
    torch = _torch()
    r = Replay(parent, n_keys, events.shape[0], queries.shape[0], blocks=blocks, chain=chain)
    answers = torch.empty(queries.shape[0], dtype=torch.int64, device=parent.device)
    r.launch(parent, events, queries, answers)
    if check:
        st = r.status()
        if st:
            raise ValueError(f"replay input rejected on the device: {STATUS_NAMES.get(st, st)}")
    return answers


def device_info():
    sms, tag = C.c_int32(0), C.c_int32(0)
    _check(gpu_lib().bw_device_info(C.byref(sms), C.byref(tag)), "bw_device_info")
    return int(sms.value), int(tag.value)
