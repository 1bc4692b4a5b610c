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
from . import shard  # noqa: F401,E402

PKG = _build.PKG

BW_EINVAL = 1001
BW_REPLAY_CHAIN_HINT = 1
BW_REPLAY_TIMING = 2
BW_REPLAY_CHAIN_KERNEL = 4
BW_REPLAY_GENERAL = 8
BW_REPLAY_WIDE = 16
PATH_FLAGS = {"auto": 0, "chain": BW_REPLAY_CHAIN_KERNEL, "general": BW_REPLAY_GENERAL}
STAGES = ["ingest", "linearise", "blocks", "prepare", "carry", "sweep"]
STATUS_NAMES = {0: "ok", 1: "events not grouped by state", 2: "event key out of range",
                3: "queries not grouped by state", 4: "query bound out of range",
                5: "bad parent array", 6: "too many key slices in a block",
                7: "state id out of range", 8: "a bounded device wait gave up"}


class BwReplayArgs(C.Structure):
    _fields_ = [("n_states", C.c_int32), ("parent", C.c_void_p), ("n_keys", C.c_uint32),
                ("n_events", C.c_int64), ("events", C.c_void_p), ("n_queries", C.c_int64),
                ("queries", C.c_void_p), ("answers", C.c_void_p), ("workspace", C.c_void_p),
                ("workspace_bytes", C.c_size_t), ("stream", C.c_void_p), ("blocks", C.c_int32),
                ("flags", C.c_int32)]


class BwCsr(C.Structure):
    _fields_ = [("key_bits", C.c_int32), ("shift", C.c_int32), ("n_buckets", C.c_int64),
                ("count", C.c_void_p), ("status", C.c_void_p), ("keys", C.c_void_p), ("pre", C.c_void_p), ("lut", C.c_void_p),
                ("low", C.c_void_p)]


class BwForestShape(C.Structure):
    _fields_ = [("n_trees", C.c_int32), ("state_off", C.c_void_p), ("event_off", C.c_void_p),
                ("query_off", C.c_void_p), ("n_keys", C.c_void_p)]


class BwForestTuning(C.Structure):
    _fields_ = [("block_work", C.c_int64), ("ctas_per_sm", C.c_int32), ("slice_ranks", C.c_int32),
                ("tile", C.c_int32), ("reserved", C.c_int32)]

    def as_dict(self) -> dict:
        return {"block_work": int(self.block_work), "ctas_per_sm": int(self.ctas_per_sm),
                "slice_ranks": int(self.slice_ranks), "tile": int(self.tile)}


class BwServeConfig(C.Structure):
    _fields_ = [("n_states", C.c_int32), ("parent", C.c_void_p), ("n_keys", C.c_uint32), ("n_events", C.c_int64),
                ("events", C.c_void_p), ("max_versions", C.c_int32), ("max_events", C.c_int64),
                ("hbm_cap_bytes", C.c_size_t), ("chain_limit", C.c_int32), ("spin_limit", C.c_uint32)]


class BwServeStats(C.Structure):
    _fields_ = [("requests", C.c_int64), ("queries", C.c_int64), ("commits", C.c_int64), ("forks", C.c_int64),
                ("wall_s", C.c_double), ("checkpoints", C.c_int32), ("spacing", C.c_int32),
                ("store_bytes", C.c_size_t), ("warps", C.c_int32), ("reserved", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: (float(getattr(self, k)) if k == "wall_s" else int(getattr(self, k)))
                for k, _ in self._fields_ if k != "reserved"}


GPU_SYMBOLS = ["gpu_v7_launch", "gpu_combine_launch", "bw_v7_carry_launch", "gpu_v7b_snap_launch",
               "gpu_v7b_launch", "gpu_v7b_combine_launch", "gpu_sess_reset_launch", "gpu_sess_run_launch",
               "gpu_sess_snap_launch", "gpu_sess_combine_launch",
               "bw_replay_workspace_size", "bw_replay_launch", "bw_replay_status",
               "bw_replay_last_info", "bw_replay_path", "bw_replay_timing_reset", "bw_replay_stage_times",
               "bw_device_info", "bw_replay_launch_noalloc",
               "bw_csr_workspace_size", "bw_csr_build", "bw_csr_point", "bw_csr_range", "bw_csr_status",
               "bw_forest_create", "bw_forest_workspace_size", "bw_forest_bind", "bw_forest_launch",
               "bw_forest_capture", "bw_forest_graph_launch", "bw_forest_status", "bw_forest_info",
               "bw_forest_destroy", "bw_forest_autotune_workspace", "bw_forest_autotune",
               "bw_forest_launch_timed",
               "bw_serve_create", "bw_serve_reset", "bw_serve_run", "bw_serve_info", "bw_serve_destroy",
               "bw_forest_plan_stats", "bw_key_histogram", "bw_key_prefix", "bw_add_range_carry",
               "bw_scatter_answers", "bw_native_expand_workspace", "bw_native_expand",
               "bw_group_workspace_size", "bw_group_events", "bw_group_queries", "bw_group_status",
               "bw_csr_events", "bw_csr_queries"]

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
        L.bw_replay_path.argtypes = [C.POINTER(BwReplayArgs), C.POINTER(C.c_int32)]
        L.bw_device_info.argtypes = [C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.bw_replay_stage_times.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_int32)]
        L.bw_v7_carry_launch.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p]
        L.gpu_v7_launch.argtypes = [C.c_void_p]
        L.gpu_combine_launch.argtypes = [C.c_void_p]
        L.bw_csr_workspace_size.argtypes = [C.c_int64, C.c_int32, C.c_size_t, C.POINTER(C.c_size_t)]
        L.bw_csr_build.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_size_t, C.c_void_p,
                                   C.c_size_t, C.c_void_p, C.POINTER(BwCsr)]
        L.bw_csr_point.argtypes = [C.POINTER(BwCsr), C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
        L.bw_csr_range.argtypes = [C.POINTER(BwCsr), C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
        L.bw_csr_status.argtypes = [C.POINTER(BwCsr), C.POINTER(C.c_int32)]
        P = C.c_void_p
        L.bw_forest_create.argtypes = [C.POINTER(BwForestShape), C.POINTER(BwForestTuning), C.POINTER(P)]
        L.bw_forest_workspace_size.argtypes = [P, C.POINTER(C.c_size_t)]
        L.bw_forest_bind.argtypes = [P, P, C.c_size_t, P]
        L.bw_forest_launch.argtypes = [P, P, P, P, P, P]
        L.bw_forest_capture.argtypes = [P, P, P, P, P, P]
        L.bw_forest_graph_launch.argtypes = [P, P]
        L.bw_forest_launch_timed.argtypes = [P, P, P, P, P, P, C.POINTER(C.c_float)]
        L.bw_serve_create.argtypes = [C.POINTER(BwServeConfig), C.POINTER(P)]
        L.bw_serve_reset.argtypes = [P]
        L.bw_serve_run.argtypes = [P, P, C.c_int64, P, C.c_int64, P, C.c_int32, C.c_double, P, P,
                                   C.POINTER(BwServeStats)]
        L.bw_serve_info.argtypes = [P, C.POINTER(BwServeStats)]
        L.bw_serve_destroy.argtypes = [P]
        L.bw_forest_status.argtypes = [P, P, C.POINTER(C.c_int32)]
        L.bw_forest_info.argtypes = [P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(BwForestTuning)]
        L.bw_forest_destroy.argtypes = [P]
        L.bw_forest_plan_stats.argtypes = [C.POINTER(BwForestShape), C.POINTER(BwForestTuning), C.c_int32,
                                           C.POINTER(C.c_int32), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
        L.bw_forest_autotune_workspace.argtypes = [C.POINTER(BwForestShape), C.POINTER(C.c_size_t)]
        L.bw_forest_autotune.argtypes = [C.POINTER(BwForestShape), P, P, P, P, P, C.c_size_t, P, C.c_int32,
                                         C.POINTER(BwForestTuning), C.POINTER(C.c_float)]
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
                 chain: bool = False, timing: bool = False, path: str = "auto", wide: bool = False,
                 device=None):
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
        a.flags = ((BW_REPLAY_CHAIN_HINT if chain else 0) | (BW_REPLAY_TIMING if timing else 0) | PATH_FLAGS[path]
                   | (BW_REPLAY_WIDE if wide else 0))
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

    def chain_path(self, events=None) -> bool:
        """Whether these arguments take the single-pass chain path (host decision)."""
        a = self.args
        if events is not None:
            a.events = events.data_ptr() if a.n_events else None
        out = C.c_int32(0)
        _check(self.lib.bw_replay_path(C.byref(a), C.byref(out)), "bw_replay_path")
        return bool(out.value)


def replay(parent, n_keys: int, events, queries, *, blocks: int = 0, chain: bool = False,
           check: bool = True, path: str = "auto", wide: bool = False):
    """One replay on the current CUDA stream; returns int64 answers on the device.
    ``path``: "auto" (the chain path for event-heavy chains with small key domains,
    else the general pipeline), "chain" or "general" to force one (chain needs
    ``chain=True``).  ``wide``: the chain path keeps an int64 histogram
    (BW_REPLAY_WIDE) -- for deltas mostly outside (-2^19, 2^19), see wide_deltas()."""
    torch = _torch()
    r = Replay(parent, n_keys, events.shape[0], queries.shape[0], blocks=blocks, chain=chain, path=path,
               wide=wide)
    answers = torch.empty(queries.shape[0], dtype=torch.int64, device=parent.device)
    r.launch(parent, events, queries, answers)
    if check:
        st = r.status()
        if st:
            raise ValueError(f"replay input rejected on the device: {STATUS_NAMES.get(st, st)}")
    return answers


def wide_deltas(events) -> bool:
    """Whether a host event array is better replayed with BW_REPLAY_WIDE: more than
    one event in 64 carries a delta outside (-2^19, 2^19) (the int32 window's range)."""
    import numpy as np
    d = np.asarray(events["delta"] if getattr(events, "dtype", None) is not None and events.dtype.names
                   else events)
    if d.size == 0:
        return False
    big = np.count_nonzero((d >= (1 << 19)) | (d <= -(1 << 19)))
    return big * 64 > d.size


class _ForestShape:
    """Host copies of a forest's offsets (kept alive while the C struct points at them)."""

    def __init__(self, state_off, event_off, query_off, n_keys):
        import numpy as np
        self.soff = np.ascontiguousarray(state_off, dtype=np.int64)
        self.eoff = np.ascontiguousarray(event_off, dtype=np.int64)
        self.qoff = np.ascontiguousarray(query_off, dtype=np.int64)
        self.keys = np.ascontiguousarray(n_keys, dtype=np.uint32)
        T = self.keys.size
        if not (self.soff.size == self.eoff.size == self.qoff.size == T + 1):
            raise ValueError("offset arrays need n_trees + 1 entries")
        self.c = BwForestShape(T, self.soff.ctypes.data, self.eoff.ctypes.data, self.qoff.ctypes.data,
                               self.keys.ctypes.data)


def _tuning(t) -> "BwForestTuning | None":
    if t is None:
        return None
    if isinstance(t, BwForestTuning):
        return t
    return BwForestTuning(int(t.get("block_work", 0)), int(t.get("ctas_per_sm", 0)), int(t.get("slice_ranks", 0)),
                          int(t.get("tile", 0)), 0)


class Forest:
    """Batched replay of many independent version trees (bw_forest_* in bw_gpu.h).

    ``state_off``/``event_off``/``query_off`` (n_trees + 1) and ``n_keys`` (n_trees)
    are host arrays; tree t's slice of the concatenated ``parent`` (int32, local ids),
    ``events`` (int64[E, 2], local states and keys) and ``queries`` (int32[Q, 3]) is a
    plain replay input.  The plan owns its device workspace (bound once)."""

    def __init__(self, state_off, event_off, query_off, n_keys, *, tuning=None, device=None, stream=None):
        torch = _torch()
        self.lib = gpu_lib()
        self.shape = _ForestShape(state_off, event_off, query_off, n_keys)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.handle = C.c_void_p()
        tu = _tuning(tuning)
        _check(self.lib.bw_forest_create(C.byref(self.shape.c), C.byref(tu) if tu is not None else None,
                                         C.byref(self.handle)), "bw_forest_create")
        nbytes = C.c_size_t(0)
        _check(self.lib.bw_forest_workspace_size(self.handle, C.byref(nbytes)), "bw_forest_workspace_size")
        self.workspace = torch.empty(max(int(nbytes.value), 256), dtype=torch.uint8, device=self.device)
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _check(self.lib.bw_forest_bind(self.handle, self.workspace.data_ptr(), self.workspace.numel(),
                                       s.cuda_stream), "bw_forest_bind")
        self.n_events = int(self.shape.eoff[-1])
        self.n_queries = int(self.shape.qoff[-1])
        self.n_states = int(self.shape.soff[-1])

    def _ptrs(self, parent, events, queries, answers):
        torch = _torch()
        if parent.dtype != torch.int32 or events.dtype != torch.int64 or queries.dtype != torch.int32 or \
                answers.dtype != torch.int64:
            raise TypeError("parent int32, events int64[E,2], queries int32[Q,3], answers int64[Q] expected")
        if parent.numel() != self.n_states or events.numel() != 2 * self.n_events or \
                queries.numel() != 3 * self.n_queries or answers.numel() != self.n_queries:
            raise ValueError("input sizes differ from the plan")
        for t in (parent, events, queries, answers):
            if not t.is_cuda or not t.is_contiguous():
                raise ValueError("inputs must be contiguous CUDA tensors")
        return (parent.data_ptr(), events.data_ptr() if self.n_events else None,
                queries.data_ptr() if self.n_queries else None, answers.data_ptr() if self.n_queries else None)

    def launch(self, parent, events, queries, answers, stream=None) -> None:
        torch = _torch()
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _check(self.lib.bw_forest_launch(self.handle, *self._ptrs(parent, events, queries, answers), s.cuda_stream),
               "bw_forest_launch")

    def launch_timed(self, parent, events, queries, answers, stream=None) -> dict:
        """One launch with CUDA events between the stages; returns per-stage ms (synchronises)."""
        torch = _torch()
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        ms = (C.c_float * len(STAGES))()
        _check(self.lib.bw_forest_launch_timed(self.handle, *self._ptrs(parent, events, queries, answers),
                                               s.cuda_stream, ms), "bw_forest_launch_timed")
        return dict(zip(STAGES, [float(x) for x in ms]))

    def capture(self, parent, events, queries, answers, stream) -> None:
        """Capture the launch with these tensors into a CUDA graph (on a non-default stream)."""
        _check(self.lib.bw_forest_capture(self.handle, *self._ptrs(parent, events, queries, answers),
                                          stream.cuda_stream), "bw_forest_capture")
        self._graph_inputs = (parent, events, queries, answers)   # keep the captured buffers alive

    def replay(self, stream=None) -> None:
        torch = _torch()
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _check(self.lib.bw_forest_graph_launch(self.handle, s.cuda_stream), "bw_forest_graph_launch")

    def status(self, stream=None) -> int:
        torch = _torch()
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        st = C.c_int32(0)
        _check(self.lib.bw_forest_status(self.handle, s.cuda_stream, C.byref(st)), "bw_forest_status")
        return int(st.value)

    def info(self) -> dict:
        b, k, tu = C.c_int32(0), C.c_int32(0), BwForestTuning()
        _check(self.lib.bw_forest_info(self.handle, C.byref(b), C.byref(k), C.byref(tu)), "bw_forest_info")
        return {"blocks": int(b.value), "kernels": int(k.value), "tuning": tu.as_dict()}

    def __del__(self):
        try:
            if self.handle:
                self.lib.bw_forest_destroy(self.handle)
                self.handle = C.c_void_p()
        except Exception:
            pass


class HostForest:
    """Replay of a forest from host buffers with the copies hidden behind the work:
    the trees are split into ``chunks`` contiguous groups of about equal events, each
    with its own plan (captured in a CUDA graph) and device buffers; chunk k+1's
    inputs are copied host to device on one stream while chunk k replays on another,
    and each chunk's answers are copied back as soon as they are ready.  Host
    buffers should be pinned (``torch.Tensor.pin_memory``) for the copies to
    overlap."""

    def __init__(self, state_off, event_off, query_off, n_keys, *, chunks: int = 4, tuning=None, device=None):
        import numpy as np
        torch = _torch()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        soff = np.asarray(state_off, dtype=np.int64)
        eoff = np.asarray(event_off, dtype=np.int64)
        qoff = np.asarray(query_off, dtype=np.int64)
        keys = np.asarray(n_keys, dtype=np.uint32)
        T = keys.size
        chunks = max(1, min(int(chunks), T))
        # cut points: equal shares of events (+ states), at tree boundaries
        weight = np.cumsum(np.diff(eoff) + np.diff(soff))
        cuts = [0] + [int(np.searchsorted(weight, weight[-1] * k / chunks)) + 1 for k in range(1, chunks)] + [T]
        cuts = sorted(set(min(max(c, 0), T) for c in cuts))
        self.copy_stream = torch.cuda.Stream(self.device)
        self.work_stream = torch.cuda.Stream(self.device)
        self.parts = []
        for a, b in zip(cuts[:-1], cuts[1:]):
            if b <= a:
                continue
            part = {"s": (int(soff[a]), int(soff[b])), "e": (int(eoff[a]), int(eoff[b])),
                    "q": (int(qoff[a]), int(qoff[b]))}
            f = Forest(soff[a:b + 1] - soff[a], eoff[a:b + 1] - eoff[a], qoff[a:b + 1] - qoff[a], keys[a:b],
                       tuning=tuning, device=self.device, stream=self.work_stream)
            ns, ne, nq = (part["s"][1] - part["s"][0], part["e"][1] - part["e"][0], part["q"][1] - part["q"][0])
            part["parent"] = torch.empty(ns, dtype=torch.int32, device=self.device)
            part["events"] = torch.empty((ne, 2), dtype=torch.int64, device=self.device)
            part["queries"] = torch.empty((nq, 3), dtype=torch.int32, device=self.device)
            part["answers"] = torch.empty(nq, dtype=torch.int64, device=self.device)
            part["forest"] = f
            part["copied"] = torch.cuda.Event()
            part["done"] = torch.cuda.Event()
            f.capture(part["parent"], part["events"], part["queries"], part["answers"], self.work_stream)
            part["done"].record(self.work_stream)
            self.parts.append(part)
        self.kernels = sum(p["forest"].info()["kernels"] for p in self.parts)

    def run(self, h_parent, h_events, h_queries, h_answers) -> None:
        """Enqueue one replay: copies in, graph launches, answers out (asynchronous;
        synchronise the device or ``self.work_stream`` before reading h_answers)."""
        cs, ws = self.copy_stream, self.work_stream
        for part in self.parts:
            (s0, s1), (e0, e1), (q0, q1) = part["s"], part["e"], part["q"]
            cs.wait_event(part["done"])          # the previous replay of this chunk is finished
            with __import__("torch").cuda.stream(cs):
                part["parent"].copy_(h_parent[s0:s1], non_blocking=True)
                part["events"].copy_(h_events[e0:e1], non_blocking=True)
                part["queries"].copy_(h_queries[q0:q1], non_blocking=True)
            part["copied"].record(cs)
            ws.wait_event(part["copied"])
            part["forest"].replay(ws)
            with __import__("torch").cuda.stream(ws):
                h_answers[q0:q1].copy_(part["answers"], non_blocking=True)
            part["done"].record(ws)

    def status(self) -> int:
        for part in self.parts:
            st = part["forest"].status(self.work_stream)
            if st:
                return st
        return 0


def forest_plan_stats(state_off, event_off, query_off, n_keys, *, tuning=None, sms: int = 152) -> dict:
    """Host-only planning of a forest (no GPU needed): blocks, workspace and carry bytes."""
    lib = gpu_lib()
    shape = _ForestShape(state_off, event_off, query_off, n_keys)
    tu = _tuning(tuning)
    b, ws, cb = C.c_int32(0), C.c_size_t(0), C.c_size_t(0)
    _check(lib.bw_forest_plan_stats(C.byref(shape.c), C.byref(tu) if tu is not None else None, int(sms), C.byref(b),
                                    C.byref(ws), C.byref(cb)), "bw_forest_plan_stats")
    return {"blocks": int(b.value), "workspace_bytes": int(ws.value), "carry_bytes": int(cb.value)}


def forest_autotune(state_off, event_off, query_off, n_keys, parent, events, queries, answers, *, reps: int = 3,
                    stream=None):
    """Time the autotuner's candidate tunings on these inputs; returns (tuning dict, ms)."""
    torch = _torch()
    lib = gpu_lib()
    shape = _ForestShape(state_off, event_off, query_off, n_keys)
    nbytes = C.c_size_t(0)
    _check(lib.bw_forest_autotune_workspace(C.byref(shape.c), C.byref(nbytes)), "bw_forest_autotune_workspace")
    ws = torch.empty(max(int(nbytes.value), 256), dtype=torch.uint8, device=parent.device)
    s = stream if stream is not None else torch.cuda.current_stream(parent.device)
    best, ms = BwForestTuning(), C.c_float(0)
    _check(lib.bw_forest_autotune(C.byref(shape.c), parent.data_ptr(), events.data_ptr() if events.numel() else None,
                                  queries.data_ptr() if queries.numel() else None,
                                  answers.data_ptr() if answers.numel() else None, ws.data_ptr(), ws.numel(),
                                  s.cuda_stream, int(reps), C.byref(best), C.byref(ms)), "bw_forest_autotune")
    return best.as_dict(), float(ms.value)


def forest_replay(state_off, event_off, query_off, n_keys, parent, events, queries, *, tuning=None,
                  check: bool = True):
    """One batched replay on the current stream; returns int64 answers on the device."""
    torch = _torch()
    f = Forest(state_off, event_off, query_off, n_keys, tuning=tuning, device=parent.device)
    answers = torch.empty(f.n_queries, dtype=torch.int64, device=parent.device)
    f.launch(parent, events, queries, answers)
    if check:
        st = f.status()
        if st:
            raise ValueError(f"forest input rejected on the device: {STATUS_NAMES.get(st, st)}")
    return answers


REQ_QUERY, REQ_COMMIT, REQ_FORK = 0, 1, 2


class Server:
    """Device-resident version store with a persistent request loop (bw_serve_* in
    bw_gpu.h).  Built from an initial tree given as host numpy arrays (parent int32,
    events EVENT_DTYPE grouped by state); requests are ``workloads.REQUEST_DTYPE``
    records served with open-loop arrival times."""

    def __init__(self, parent, n_keys: int, events, *, max_versions: int, max_events: int,
                 hbm_cap_bytes: int, chain_limit: int = 0, spin_limit: int = 0):
        import numpy as np
        _torch()
        self.lib = gpu_lib()
        par = np.ascontiguousarray(parent, dtype=np.int32)
        ev = np.ascontiguousarray(events)
        if ev.dtype != workloads.EVENT_DTYPE:
            raise TypeError("events must be workloads.EVENT_DTYPE records")
        cfg = BwServeConfig(int(par.size), par.ctypes.data, int(n_keys), int(ev.size),
                            ev.ctypes.data if ev.size else None, int(max_versions), int(max_events),
                            int(hbm_cap_bytes), int(chain_limit), int(spin_limit))
        self.handle = C.c_void_p()
        _check(self.lib.bw_serve_create(C.byref(cfg), C.byref(self.handle)), "bw_serve_create")
        self.n_keys = int(n_keys)
        self.n_states = int(par.size)

    def info(self) -> dict:
        st = BwServeStats()
        _check(self.lib.bw_serve_info(self.handle, C.byref(st)), "bw_serve_info")
        return st.as_dict()

    def reset(self) -> None:
        _check(self.lib.bw_serve_reset(self.handle), "bw_serve_reset")

    def run(self, requests, commit_events=None, arrival_s=None, *, max_inflight: int = 1 << 16,
            timeout_s: float = 300.0):
        """Serve a request log; returns (answers int64[n], latency_us float32[n], stats dict)."""
        import numpy as np
        req = np.ascontiguousarray(requests)
        if req.dtype != workloads.REQUEST_DTYPE:
            raise TypeError("requests must be workloads.REQUEST_DTYPE records")
        cev = np.ascontiguousarray(commit_events if commit_events is not None
                                   else np.empty(0, dtype=workloads.EVENT_DTYPE))
        arr = None if arrival_s is None else np.ascontiguousarray(arrival_s, dtype=np.float64)
        if arr is not None and arr.size != req.size:
            raise ValueError("one arrival time per request")
        n = int(req.size)
        answers = np.zeros(n, dtype=np.int64)
        lat = np.zeros(n, dtype=np.float32)
        st = BwServeStats()
        _check(self.lib.bw_serve_run(self.handle, req.ctypes.data if n else None, n,
                                     cev.ctypes.data if cev.size else None, int(cev.size),
                                     arr.ctypes.data if arr is not None else None, int(max_inflight),
                                     float(timeout_s), answers.ctypes.data if n else None,
                                     lat.ctypes.data if n else None, C.byref(st)), "bw_serve_run")
        return answers, lat, st.as_dict()

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.bw_serve_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def device_info():
    sms, tag = C.c_int32(0), C.c_int32(0)
    _check(gpu_lib().bw_device_info(C.byref(sms), C.byref(tag)), "bw_device_info")
    return int(sms.value), int(tag.value)


# ---------------------------------------------------------------------------- host side
class BwNativeSpec(C.Structure):
    _fields_ = [("n_states", C.c_int32), ("topology", C.c_int32), ("seed", C.c_int32),
                ("factor_period", C.c_int32), ("q", C.c_int32), ("per_state", C.c_int32),
                ("factor_pct", C.c_int32)]


class BwNativeWorkload(C.Structure):
    _fields_ = [("n_states", C.c_int32), ("n_keys", C.c_uint32), ("n_events", C.c_int64),
                ("n_queries", C.c_int64), ("parent", C.c_void_p), ("events", C.c_void_p),
                ("queries", C.c_void_p), ("n_factor_events", C.c_int64)]


HOST_SYMBOLS = ["bw_fixture_open", "bw_fixture_from_memory", "bw_fixture_close", "bw_fixture_rows",
                "bw_native_build", "bw_native_free", "bw_native_build_declared", "bw_v7_plan_build",
                "bw_v7_plan_build_declared", "bw_v7_plan_free", "bw_sha256_hex", "bw_fnv1a",
                "bw_sha256_init", "bw_sha256_update", "bw_sha256_final", "bw_fnv1a_update",
                "bw_stream_build", "bw_stream_free", "bw_native_build_compact", "bw_native_compact_free"]

_host = None


def host_lib(build_if_missing: bool = True):
    """The host C++ library (fixtures, declared workloads, digests)."""
    global _host
    if _host is None:
        if build_if_missing:
            _build.build()
        L = C.CDLL(str(_build.HOST_LIB))
        L.bw_fixture_from_memory.argtypes = [C.c_void_p, C.c_size_t, C.POINTER(C.c_void_p)]
        L.bw_fixture_open.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
        L.bw_fixture_close.argtypes = [C.c_void_p]
        L.bw_fixture_rows.argtypes = [C.c_void_p]
        L.bw_fixture_rows.restype = C.c_int64
        L.bw_native_build.argtypes = [C.c_void_p, C.POINTER(BwNativeSpec),
                                      C.POINTER(C.POINTER(BwNativeWorkload))]
        L.bw_native_free.argtypes = [C.POINTER(BwNativeWorkload)]
        L.bw_sha256_hex.argtypes = [C.c_void_p, C.c_size_t, C.c_char_p]
        L.bw_fnv1a.argtypes = [C.c_void_p, C.c_size_t]
        L.bw_fnv1a.restype = C.c_uint64
        L.bw_sha256_init.argtypes = [C.c_void_p]
        L.bw_sha256_update.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
        L.bw_sha256_final.argtypes = [C.c_void_p, C.c_char_p]
        L.bw_fnv1a_update.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
        L.bw_fnv1a_update.restype = C.c_uint64
        _host = L
    return _host


def sha256_hex(buf) -> str:
    import numpy as np
    a = np.ascontiguousarray(np.frombuffer(memoryview(buf).cast("B"), dtype=np.uint8))
    out = C.create_string_buffer(65)
    host_lib().bw_sha256_hex(a.ctypes.data if a.size else None, a.size, out)
    return out.value.decode()


def fnv1a(buf) -> int:
    import numpy as np
    a = np.ascontiguousarray(np.frombuffer(memoryview(buf).cast("B"), dtype=np.uint8))
    return int(host_lib().bw_fnv1a(a.ctypes.data if a.size else None, a.size))


class Digest:
    """Streaming SHA-256 + FNV-1a over bytes fed in pieces (bw_sha256_update,
    bw_fnv1a_update): the worker's extract digests each downloaded chunk this way."""

    FNV_BASIS = 1469598103934665603

    def __init__(self):
        self._state = C.create_string_buffer(256)   # a BwSha256 (128 bytes), with room to spare
        host_lib().bw_sha256_init(self._state)
        self._fnv = self.FNV_BASIS

    def update(self, buf) -> None:
        import numpy as np
        a = np.ascontiguousarray(np.frombuffer(memoryview(buf).cast("B"), dtype=np.uint8))
        ptr = a.ctypes.data if a.size else None
        host_lib().bw_sha256_update(self._state, ptr, a.size)
        self._fnv = int(host_lib().bw_fnv1a_update(self._fnv, ptr, a.size))

    def final(self):
        out = C.create_string_buffer(65)
        host_lib().bw_sha256_final(self._state, out)
        return out.value.decode(), self._fnv


class BwDeclared(C.Structure):
    _fields_ = [("n_states", C.c_int32), ("q", C.c_int32), ("per_state", C.c_int32), ("parent", C.c_void_p),
                ("op", C.c_void_p), ("g", C.c_void_p), ("id", C.c_void_p), ("val", C.c_void_p), ("t", C.c_void_p),
                ("qlo", C.c_void_p), ("qhi", C.c_void_p), ("n_inserted", C.c_int64), ("ins_t", C.c_void_p),
                ("ins_g", C.c_void_p)]


def _declared(decl):
    """A BwDeclared over numpy copies of ``decl``'s arrays (kept alive with it)."""
    import numpy as np
    keep = {"parent": np.ascontiguousarray(decl.parent, np.int32), "op": np.ascontiguousarray(decl.op, np.uint8),
            "g": np.ascontiguousarray(decl.g, np.int32), "id": np.ascontiguousarray(decl.id, np.int64),
            "val": np.ascontiguousarray(decl.val, np.int64), "t": np.ascontiguousarray(decl.t, np.int64),
            "qlo": np.ascontiguousarray(decl.qlo, np.int64), "qhi": np.ascontiguousarray(decl.qhi, np.int64),
            "ins_t": np.ascontiguousarray(decl.ins_t, np.int64).reshape(-1),
            "ins_g": np.ascontiguousarray(decl.ins_g, np.int32).reshape(-1)}
    d = BwDeclared()
    d.n_states, d.q, d.per_state = int(keep["parent"].size), int(decl.q), int(bool(decl.per_state))
    d.n_inserted = int(keep["ins_t"].size)
    for k, a in keep.items():
        setattr(d, k, a.ctypes.data if a.size else None)
    return d, keep


def _with_fixture(fixture: bytes, fn):
    import numpy as np
    L = host_lib()
    img = np.frombuffer(fixture, dtype=np.uint8)
    fx = C.c_void_p()
    rc = L.bw_fixture_from_memory(img.ctypes.data, img.size, C.byref(fx))
    if rc:
        raise ValueError(f"malformed BWBASE02 fixture (rc={rc})")
    try:
        return fn(L, fx)
    finally:
        L.bw_fixture_close(fx)


def _native_result(L, out, name: str, chain: bool) -> "workloads.Workload":
    import numpy as np
    try:
        w = out.contents
        S, E, Q = w.n_states, w.n_events, w.n_queries
        parent = np.ctypeslib.as_array(C.cast(w.parent, C.POINTER(C.c_int32)), (S,)).copy()
        ev = np.frombuffer(C.string_at(w.events, 16 * E), dtype=workloads.EVENT_DTYPE).copy() \
            if E else np.empty(0, dtype=workloads.EVENT_DTYPE)
        qs = np.frombuffer(C.string_at(w.queries, 12 * Q), dtype=workloads.QUERY_DTYPE).copy() \
            if Q else np.empty(0, dtype=workloads.QUERY_DTYPE)
        return workloads.Workload(name, parent, int(w.n_keys), ev, qs, chain)
    finally:
        L.bw_native_free(out)


def native_workload(fixture: bytes, n_states: int, topology: int, seed: int, factor_period: int,
                    q: int, per_state: bool = True, factor_pct: int = -1) -> "workloads.Workload":
    """Compile a reference-native case (BWBASE02 image + declared edits) into the
    event model: class-delta events by state and class-interval queries in the
    reference's answer order (v = 1..S-1, k = 0..q-1)."""
    def run(L, fx):
        spec = BwNativeSpec(n_states, topology, seed, factor_period, q, int(per_state), factor_pct)
        out = C.POINTER(BwNativeWorkload)()
        rc = L.bw_native_build(fx, C.byref(spec), C.byref(out))
        if rc:
            raise ValueError(f"native workload rejected (rc={rc})")
        return _native_result(L, out, f"native_S{n_states}_t{topology}_s{seed}_f{factor_period}_q{q}", topology == 0)
    return _with_fixture(fixture, run)


def native_workload_declared(fixture: bytes, decl, name: str = "declared") -> "workloads.Workload":
    """The event model of an explicit declared workload (bw_native_build_declared):
    ``decl`` carries n-state arrays parent/op/g/id/val/t, declared ranges qlo/qhi,
    inserted rows ins_t/ins_g, q and per_state (the reference fuzz's Workload)."""
    import numpy as np

    def run(L, fx):
        L.bw_native_build_declared.argtypes = [C.c_void_p, C.POINTER(BwDeclared),
                                               C.POINTER(C.POINTER(BwNativeWorkload))]
        d, _keep = _declared(decl)
        out = C.POINTER(BwNativeWorkload)()
        rc = L.bw_native_build_declared(fx, C.byref(d), C.byref(out))
        if rc:
            raise ValueError(f"declared workload rejected (rc={rc})")
        par = np.asarray(decl.parent)
        chain = bool(np.all(par[1:] == np.arange(par.size - 1)))
        return _native_result(L, out, name, chain)
    return _with_fixture(fixture, run)


class BwTimeline(C.Structure):
    _fields_ = [("state", C.c_int32), ("idx", C.c_int32), ("value", C.c_int64), ("out", C.c_int64)]


class BwNativeCompact(C.Structure):
    _fields_ = [("n_states", C.c_int32), ("n_groups", C.c_int32), ("n_keys", C.c_uint32), ("n_events", C.c_int64),
                ("n_queries", C.c_int64), ("parent", C.c_void_p), ("queries", C.c_void_p), ("n_fixed", C.c_int64),
                ("fixed", C.c_void_p), ("fixed_pos", C.c_void_p), ("sup_off", C.c_void_p), ("sup_cls", C.c_void_p),
                ("base_mass", C.c_void_p), ("tl_off", C.c_void_p), ("tl", C.POINTER(BwTimeline))]


def native_compact(fixture: bytes, n_states: int, seed: int, factor_period: int, q: int, per_state: bool = True,
                   factor_pct: int = -1) -> dict:
    """The compact form of a reference-native chain (bw_native_build_compact) as numpy
    arrays: verbatim events and their positions, group supports and base masses,
    per-group timelines (mass updates, factor expansions)."""
    import numpy as np

    def run(L, fx):
        L.bw_native_build_compact.argtypes = [C.c_void_p, C.POINTER(BwNativeSpec),
                                              C.POINTER(C.POINTER(BwNativeCompact))]
        L.bw_native_compact_free.argtypes = [C.POINTER(BwNativeCompact)]
        spec = BwNativeSpec(n_states, 0, seed, factor_period, q, int(per_state), factor_pct)
        out = C.POINTER(BwNativeCompact)()
        rc = L.bw_native_build_compact(fx, C.byref(spec), C.byref(out))
        if rc:
            raise ValueError(f"compact chain build rejected (rc={rc})")
        try:
            c = out.contents
            G = c.n_groups

            def arr(ptr, dtype, n):
                n = int(n)
                return np.frombuffer(C.string_at(ptr, np.dtype(dtype).itemsize * n), dtype=dtype).copy() if n else \
                    np.empty(0, dtype=dtype)
            sup_off = arr(c.sup_off, np.int64, G + 1)
            tl_off = arr(c.tl_off, np.int64, G + 1)
            tl_dt = np.dtype([("state", "<i4"), ("idx", "<i4"), ("value", "<i8"), ("out", "<i8")])
            return {"n_states": c.n_states, "n_groups": G, "n_keys": int(c.n_keys), "n_events": int(c.n_events),
                    "parent": arr(c.parent, np.int32, c.n_states),
                    "queries": arr(c.queries, workloads.QUERY_DTYPE, c.n_queries),
                    "fixed": arr(c.fixed, workloads.EVENT_DTYPE, c.n_fixed),
                    "fixed_pos": arr(c.fixed_pos, np.int64, c.n_fixed), "sup_off": sup_off,
                    "sup_cls": arr(c.sup_cls, np.uint32, sup_off[-1]),
                    "base_mass": arr(c.base_mass, np.int64, sup_off[-1]), "tl_off": tl_off,
                    "tl": arr(C.cast(c.tl, C.c_void_p), tl_dt, tl_off[-1])}
        finally:
            L.bw_native_compact_free(out)
    return _with_fixture(fixture, run)


def expand_events(compact: dict, device=None):
    """The compact chain's events on the device (bw_native_expand): an (n_events, 2)
    int64 tensor, grouped by state."""
    import numpy as np
    torch = _torch()
    L = gpu_lib()
    L.bw_native_expand_workspace.argtypes = [C.POINTER(BwNativeCompact), C.POINTER(C.c_size_t)]
    L.bw_native_expand.argtypes = [C.POINTER(BwNativeCompact), C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    keep = {k: np.ascontiguousarray(v) for k, v in compact.items() if isinstance(v, np.ndarray)}
    c = BwNativeCompact()
    c.n_states, c.n_groups, c.n_keys = compact["n_states"], compact["n_groups"], compact["n_keys"]
    c.n_events, c.n_queries = compact["n_events"], len(keep["queries"])
    c.n_fixed = len(keep["fixed"])

    def ptr(k):
        return keep[k].ctypes.data if keep[k].size else None
    c.parent, c.queries, c.fixed, c.fixed_pos = ptr("parent"), ptr("queries"), ptr("fixed"), ptr("fixed_pos")
    c.sup_off, c.sup_cls, c.base_mass, c.tl_off = ptr("sup_off"), ptr("sup_cls"), ptr("base_mass"), ptr("tl_off")
    c.tl = C.cast(ptr("tl"), C.POINTER(BwTimeline))
    need = C.c_size_t(0)
    _check(L.bw_native_expand_workspace(C.byref(c), C.byref(need)), "bw_native_expand_workspace")
    dev = device or torch.device("cuda")
    ws = torch.empty(max(int(need.value), 256), dtype=torch.uint8, device=dev)
    ev = torch.empty((max(compact["n_events"], 1), 2), dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)
    _check(L.bw_native_expand(C.byref(c), ev.data_ptr(), ws.data_ptr(), ws.numel(), stream.cuda_stream),
           "bw_native_expand")
    stream.synchronize()   # the host arrays are only needed until the copies are done
    return ev[:compact["n_events"]]


def group_by_state(n_states: int, events=None, queries=None, check: bool = True):
    """Group device event and/or query arrays by state (bw_group_events,
    bw_group_queries): a stable radix sort on the state.  Returns (events, queries,
    order): the grouped copies and, for queries, order[i] = the input index of grouped
    query i (scatter_device_answers puts answers back in input order)."""
    torch = _torch()
    L = gpu_lib()
    L.bw_group_workspace_size.argtypes = [C.c_int64, C.c_int32, C.POINTER(C.c_size_t)]
    L.bw_group_events.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    L.bw_group_queries.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_size_t, C.c_void_p]
    L.bw_group_status.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
    out_e = out_q = order = None
    for kind, arr in (("events", events), ("queries", queries)):
        if arr is None:
            continue
        n = int(arr.shape[0])
        need = C.c_size_t(0)
        _check(L.bw_group_workspace_size(n, int(kind == "queries"), C.byref(need)), "bw_group_workspace_size")
        ws = torch.empty(max(int(need.value), 256), dtype=torch.uint8, device=arr.device)
        stream = torch.cuda.current_stream(arr.device).cuda_stream
        if kind == "events":
            out_e = torch.empty_like(arr)
            _check(L.bw_group_events(arr.data_ptr(), n, int(n_states), out_e.data_ptr(), ws.data_ptr(), ws.numel(),
                                     stream), "bw_group_events")
        else:
            out_q = torch.empty_like(arr)
            order = torch.empty(max(n, 1), dtype=torch.int64, device=arr.device)[:n]
            _check(L.bw_group_queries(arr.data_ptr(), n, int(n_states), out_q.data_ptr(), order.data_ptr(),
                                      ws.data_ptr(), ws.numel(), stream), "bw_group_queries")
        if check and n:
            st = C.c_int32(0)
            _check(L.bw_group_status(ws.data_ptr(), C.byref(st)), "bw_group_status")
            if st.value:
                raise ValueError(f"{kind} rejected on the device: {STATUS_NAMES.get(st.value, st.value)}")
    return out_e, out_q, order


def scatter_device_answers(answers, slot, n_out: int):
    """out[slot[i]] = answers[i] on the device (bw_scatter_answers)."""
    torch = _torch()
    L = gpu_lib()
    L.bw_scatter_answers.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]
    out = torch.zeros(max(n_out, 1), dtype=torch.int64, device=answers.device)[:n_out]
    _check(L.bw_scatter_answers(answers.data_ptr(), slot.data_ptr(), int(answers.numel()), out.data_ptr(), n_out,
                                torch.cuda.current_stream(answers.device).cuda_stream), "bw_scatter_answers")
    return out


def versioned_sparse_replay(parent, ev_state, ev_key, ev_delta, q_state, lo, hi=None, *, key_bits: int = 40,
                            lut_budget_bytes: int = 64 << 20, index=None, path: str = "auto"):
    """A version tree over sparse u64 keys (config 3's versioned dimension): the keys'
    CSR rank index on the device (bw_csr_build, or `index`), events and lookups mapped
    to ranks there (bw_csr_events, bw_csr_queries), then the replay over the rank
    domain.  Point lookups when hi is None, else range lookups over [lo, hi).
    Returns (answers, index)."""
    idx = index if index is not None else CsrIndex(ev_key, ev_delta, key_bits=key_bits,
                                                   lut_budget_bytes=lut_budget_bytes)
    ev = idx.events(ev_state, ev_key, ev_delta)
    qs = idx.queries(q_state, lo, hi)
    return replay(parent, max(1, idx.count()), ev, qs, path=path), idx


class BwStreamWorkload(C.Structure):
    _fields_ = [("chain", BwNativeWorkload), ("slot", C.c_void_p), ("n_answers", C.c_int64), ("q", C.c_int32)]


def stream_workload(fixture: bytes, stream: bytes, name: str = "stream"):
    """The reference's BWLEV001 event stream (emit_events.cpp) over a BWBASE02 fixture,
    compiled into a linear-chain event workload (bw_stream_build).  Returns
    (workload, slot, n_answers): answers of the chain queries, scattered by ``slot``
    (-1: not in the answer vector), give the reference's answer vector."""
    import numpy as np

    def run(L, fx):
        L.bw_stream_build.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t, C.POINTER(C.POINTER(BwStreamWorkload))]
        L.bw_stream_free.argtypes = [C.POINTER(BwStreamWorkload)]
        out = C.POINTER(BwStreamWorkload)()
        rc = L.bw_stream_build(fx, stream, len(stream), C.byref(out))
        if rc:
            raise ValueError(f"event stream rejected (rc={rc})")
        try:
            o = out.contents
            w = o.chain
            S, E, Q = w.n_states, w.n_events, w.n_queries
            parent = np.ctypeslib.as_array(C.cast(w.parent, C.POINTER(C.c_int32)), (S,)).copy()
            ev = np.frombuffer(C.string_at(w.events, 16 * E), dtype=workloads.EVENT_DTYPE).copy() \
                if E else np.empty(0, dtype=workloads.EVENT_DTYPE)
            qs = np.frombuffer(C.string_at(w.queries, 12 * Q), dtype=workloads.QUERY_DTYPE).copy() \
                if Q else np.empty(0, dtype=workloads.QUERY_DTYPE)
            slot = np.frombuffer(C.string_at(o.slot, 8 * Q), dtype=np.int64).copy() if Q else \
                np.empty(0, dtype=np.int64)
            return workloads.Workload(name, parent, int(w.n_keys), ev, qs, True), slot, int(o.n_answers)
        finally:
            L.bw_stream_free(out)
    return _with_fixture(fixture, run)


def scatter_answers(chain_answers, slot, n_answers):
    """The answer vector from a stream workload's chain answers (stream order)."""
    import numpy as np
    out = np.zeros(n_answers, dtype=np.int64)
    keep = slot >= 0
    out[slot[keep]] = np.asarray(chain_answers)[keep]
    return out


class BwV7Plan(C.Structure):
    _fields_ = [("B", C.c_int32), ("G", C.c_int32), ("Cpfx", C.c_int32), ("ncls", C.c_int32),
                ("q", C.c_int32), ("n_states", C.c_int32), ("n_active", C.c_int32),
                ("nodes", C.c_void_p), ("block_v0", C.c_void_p), ("block_v1", C.c_void_p),
                ("fac_start", C.c_void_p), ("g2row", C.c_void_p), ("ms_off", C.c_void_p),
                ("ms_cls", C.c_void_p), ("ms_base", C.c_void_p), ("ms_dev", C.c_void_p),
                ("devbuf", C.c_void_p), ("n_devbuf", C.c_int64), ("need_off", C.c_void_p),
                ("qlb", C.c_void_p), ("qhb", C.c_void_p), ("bidx", C.c_void_p), ("vbase", C.c_void_p)]


def _node_dtype():
    import numpy as np
    return np.dtype([("kind", "<i4"), ("g_old", "<i4"), ("c_old", "<i4"), ("ti_old", "<i4"),
                     ("g_new", "<i4"), ("c_new", "<i4"), ("ti_new", "<i4"), ("pad0", "<i4"),
                     ("amt_old", "<i8"), ("amt_new", "<i8"), ("fac_val", "<i8"), ("fac_prev", "<i8"),
                     ("ex_old", "u1"), ("ex_new", "u1"), ("pad", "u1", (6,))])


def _v7_result(L, out) -> dict:
    import numpy as np
    try:
        p = out.contents
        B, G, Cp, S, na = p.B, p.G, p.Cpfx, p.n_states, p.n_active

        def arr(ptr, dtype, n):
            dt = np.dtype(dtype)
            return np.frombuffer(C.string_at(ptr, dt.itemsize * n), dtype=dt).copy() if n else np.zeros(0, dt)
        ms_off = arr(p.ms_off, "<i4", na + 1)
        nms = int(ms_off[-1])
        return {"B": B, "G": G, "Cpfx": Cp, "ncls": p.ncls, "q": p.q, "n_states": S,
                "nodes": arr(p.nodes, _node_dtype(), S), "block_v0": arr(p.block_v0, "<i4", B),
                "block_v1": arr(p.block_v1, "<i4", B), "fac_start": arr(p.fac_start, "<i8", B * G),
                "g2row": arr(p.g2row, "<i4", G), "ms_off": ms_off, "ms_cls": arr(p.ms_cls, "<i8", nms),
                "ms_base": arr(p.ms_base, "<i8", nms), "ms_dev": arr(p.ms_dev, "<i4", nms),
                "devbuf": arr(p.devbuf, "<i8", max(1, p.n_devbuf)), "need_off": arr(p.need_off, "<i8", B * G),
                "qlb": arr(p.qlb, "<i4", S * p.q), "qhb": arr(p.qhb, "<i4", S * p.q),
                "bidx": arr(p.bidx, "<i4", S), "vbase": arr(p.vbase, "<i8", Cp)}
    finally:
        L.bw_v7_plan_free(out)


def v7_plan(fixture: bytes, n_states: int, seed: int, factor_period: int, q: int, blocks: int,
            per_state: bool = True, factor_pct: int = -1) -> dict:
    """The reference's v7 chain plan for gpu_v7_launch, as numpy arrays."""
    def run(L, fx):
        L.bw_v7_plan_build.argtypes = [C.c_void_p, C.POINTER(BwNativeSpec), C.c_int32,
                                       C.POINTER(C.POINTER(BwV7Plan))]
        L.bw_v7_plan_free.argtypes = [C.POINTER(BwV7Plan)]
        spec = BwNativeSpec(n_states, 0, seed, factor_period, q, int(per_state), factor_pct)
        out = C.POINTER(BwV7Plan)()
        rc = L.bw_v7_plan_build(fx, C.byref(spec), blocks, C.byref(out))
        if rc:
            raise ValueError(f"v7 plan rejected (rc={rc})")
        return _v7_result(L, out)
    return _with_fixture(fixture, run)


def v7_plan_declared(fixture: bytes, decl, blocks: int) -> dict:
    """The v7 chain plan of an explicit declared chain workload (bw_v7_plan_build_declared)."""
    def run(L, fx):
        L.bw_v7_plan_build_declared.argtypes = [C.c_void_p, C.POINTER(BwDeclared), C.c_int32,
                                                C.POINTER(C.POINTER(BwV7Plan))]
        L.bw_v7_plan_free.argtypes = [C.POINTER(BwV7Plan)]
        d, _keep = _declared(decl)
        out = C.POINTER(BwV7Plan)()
        rc = L.bw_v7_plan_build_declared(fx, C.byref(d), blocks, C.byref(out))
        if rc:
            raise ValueError(f"v7 plan rejected (rc={rc})")
        return _v7_result(L, out)
    return _with_fixture(fixture, run)


class GpuV7Args(C.Structure):
    _fields_ = [("B", C.c_int), ("G", C.c_int), ("Cpfx", C.c_int), ("ncls", C.c_int), ("q", C.c_int),
                ("nodes", C.c_void_p), ("block_v0", C.c_void_p), ("block_v1", C.c_void_p),
                ("fac_start", C.c_void_p), ("g2row", C.c_void_p), ("ms_off", C.c_void_p),
                ("ms_cls", C.c_void_p), ("ms_base", C.c_void_p), ("ms_dev", C.c_void_p),
                ("devbuf", C.c_void_p), ("need_off", C.c_void_p), ("qlb", C.c_void_p), ("qhb", C.c_void_p),
                ("lvals", C.c_void_p), ("dV", C.c_void_p), ("threads", C.c_int), ("shared_bytes", C.c_int)]


class GpuV7CombineArgs(C.Structure):
    _fields_ = [("nstates", C.c_int), ("q", C.c_int), ("Cpfx", C.c_int), ("qlb", C.c_void_p),
                ("qhb", C.c_void_p), ("carrypref", C.c_void_p), ("bidx", C.c_void_p),
                ("lvals", C.c_void_p), ("answers", C.c_void_p)]


def run_v7_plan(plan: dict):
    """Drive the drop-in gpu_v7 ABI exactly as the reference worker does
    (panel_batch_gpu.cpp:171-224): block kernel, carry, combine.  The carry runs
    on the device (bw_v7_carry_launch) instead of the host.  Returns answers."""
    import numpy as np
    torch = _torch()
    L = gpu_lib()
    dev = torch.device("cuda")

    def up(a):
        return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8)).to(dev)
    d = {k: up(plan[k]) for k in ("nodes", "block_v0", "block_v1", "fac_start", "g2row", "ms_off", "ms_cls",
                                  "ms_base", "ms_dev", "devbuf", "need_off", "qlb", "qhb", "bidx", "vbase")}
    B, Cp, q, S = plan["B"], plan["Cpfx"], plan["q"], plan["n_states"]
    lvals = torch.empty((S - 1) * 2 * q, dtype=torch.int64, device=dev)
    dV = torch.empty(B * Cp, dtype=torch.int64, device=dev)
    carry = torch.empty(B * Cp, dtype=torch.int64, device=dev)
    answers = torch.empty((S - 1) * q, dtype=torch.int64, device=dev)
    a = GpuV7Args(B, plan["G"], Cp, plan["ncls"], q, *(d[k].data_ptr() for k in (
        "nodes", "block_v0", "block_v1", "fac_start", "g2row", "ms_off", "ms_cls", "ms_base", "ms_dev",
        "devbuf", "need_off", "qlb", "qhb")), lvals.data_ptr(), dV.data_ptr(), 256, 0)
    torch.cuda.synchronize()
    _check(L.gpu_v7_launch(C.byref(a)), "gpu_v7_launch")
    _check(L.bw_v7_carry_launch(B, Cp, d["vbase"].data_ptr(), dV.data_ptr(), carry.data_ptr(), None),
           "bw_v7_carry_launch")
    ca = GpuV7CombineArgs(S - 1, q, Cp, d["qlb"].data_ptr(), d["qhb"].data_ptr(), carry.data_ptr(),
                          d["bidx"].data_ptr(), lvals.data_ptr(), answers.data_ptr())
    _check(L.gpu_combine_launch(C.byref(ca)), "gpu_combine_launch")
    torch.cuda.synchronize()
    return answers.cpu().numpy(), dV.cpu().numpy(), lvals.cpu().numpy()


class GpuV7bArgs(C.Structure):
    _fields_ = [("B", C.c_int), ("G", C.c_int), ("Cpfx", C.c_int), ("ncls", C.c_int), ("q", C.c_int),
                ("nodes", C.c_void_p), ("bv0", C.c_void_p), ("bv1", C.c_void_p), ("fac_start", C.c_void_p),
                ("g2row", C.c_void_p), ("ms_off", C.c_void_p), ("ms_cls", C.c_void_p), ("ms_base", C.c_void_p),
                ("ms_dev", C.c_void_p), ("devbuf", C.c_void_p), ("need_off", C.c_void_p), ("qlb", C.c_void_p),
                ("qhb", C.c_void_p), ("lvals", C.c_void_p), ("dV", C.c_void_p), ("threads", C.c_int),
                ("shared_bytes", C.c_int)]


class GpuSessRunArgs(C.Structure):
    _fields_ = GpuV7bArgs._fields_[:-2] + [("fen", C.c_void_p), ("leaf", C.c_void_p), ("threads", C.c_int)]


class GpuV7bSnapArgs(C.Structure):
    _fields_ = [("nstates", C.c_int), ("nodes", C.c_void_p), ("bidx", C.c_void_p), ("gb_off", C.c_void_p),
                ("gb_block", C.c_void_p), ("gb_reg", C.c_void_p), ("devbuf", C.c_void_p)]


class GpuSessResetArgs(C.Structure):
    _fields_ = [("B", C.c_int), ("Cpfx", C.c_int), ("fen", C.c_void_p), ("leaf", C.c_void_p)]


def compact_plan(plan: dict) -> dict:
    """The v7b / session form of a v7 plan (gpu_v7b.h:6-21): 40-byte nodes (kind bits
    1 row, 2 factor, 4 ex_old, 8 ex_new; a, b = amt_old, amt_new or fac_val, fac_prev)
    and the (group, block) occurrence tables of the device snapshot entry."""
    import numpy as np
    n = plan["nodes"]
    dt = np.dtype([("kind", "u1"), ("pad0", "u1"), ("g_old", "<i2"), ("g_new", "<i2"), ("pad1", "u1", (2,)),
                   ("c_old", "<i4"), ("c_new", "<i4"), ("ti_old", "<i4"), ("ti_new", "<i4"),
                   ("a", "<i8"), ("b", "<i8")])
    assert dt.itemsize == 40
    cn = np.zeros(n.size, dtype=dt)
    row, fac = n["kind"] == 1, n["kind"] == 2
    cn["kind"] = n["kind"] | (n["ex_old"].astype(np.int32) << 2) | (n["ex_new"].astype(np.int32) << 3)
    cn["g_old"], cn["g_new"] = n["g_old"], n["g_new"]
    cn["c_old"], cn["c_new"], cn["ti_old"], cn["ti_new"] = n["c_old"], n["c_new"], n["ti_old"], n["ti_new"]
    cn["a"] = np.where(row, n["amt_old"], np.where(fac, n["fac_val"], 0))
    cn["b"] = np.where(row, n["amt_new"], np.where(fac, n["fac_prev"], 0))
    B, G = plan["B"], plan["G"]
    need = plan["need_off"].reshape(B, G)
    gb_off, gb_block, gb_reg = [0], [], []
    for g in range(G):
        bs = np.nonzero(need[:, g] >= 0)[0]
        gb_block += bs.tolist()
        gb_reg += need[bs, g].tolist()
        gb_off.append(len(gb_block))
    return {"nodes": cn, "gb_off": np.array(gb_off, np.int32), "gb_block": np.array(gb_block or [0], np.int32),
            "gb_reg": np.array(gb_reg or [0], np.int64)}


def run_v7b_plan(plan: dict, session: bool = False, batches: int = 1):
    """Drive the compact drop-in ABI as the reference's snapshot worker (gpu_v7b.h,
    panel_batch_gpu2.cpp:193-244) or session worker (gpu_session.h,
    panel_gpu_session.cpp:110-137) do: device snapshots into a zeroed devbuf, block
    replay (session: reset + run per batch, prefix structure in global memory), carry,
    combine.  Returns (answers, devbuf after the snapshot entry)."""
    import numpy as np
    torch = _torch()
    L = gpu_lib()
    dev = torch.device("cuda")
    cp = compact_plan(plan)

    def up(a):
        return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8)).to(dev)
    d = {k: up(plan[k]) for k in ("block_v0", "block_v1", "fac_start", "g2row", "ms_off", "ms_cls", "ms_base",
                                  "ms_dev", "need_off", "qlb", "qhb", "bidx", "vbase")}
    d.update({k: up(cp[k]) for k in ("nodes", "gb_off", "gb_block", "gb_reg")})
    B, Cp, q, S, G = plan["B"], plan["Cpfx"], plan["q"], plan["n_states"], plan["G"]
    devbuf = torch.zeros(max(1, plan["devbuf"].size), dtype=torch.int64, device=dev)
    lvals = torch.empty((S - 1) * 2 * q, dtype=torch.int64, device=dev)
    dV = torch.empty(B * Cp, dtype=torch.int64, device=dev)
    carry = torch.empty(B * Cp, dtype=torch.int64, device=dev)
    answers = torch.empty((S - 1) * q, dtype=torch.int64, device=dev)
    torch.cuda.synchronize()
    sa = GpuV7bSnapArgs(S, d["nodes"].data_ptr(), d["bidx"].data_ptr(), d["gb_off"].data_ptr(),
                        d["gb_block"].data_ptr(), d["gb_reg"].data_ptr(), devbuf.data_ptr())
    for name in ("gpu_v7b_snap_launch", "gpu_sess_snap_launch", "gpu_v7b_launch", "gpu_sess_run_launch",
                 "gpu_sess_reset_launch", "gpu_v7b_combine_launch", "gpu_sess_combine_launch"):
        getattr(L, name).argtypes = [C.c_void_p]
    _check((L.gpu_sess_snap_launch if session else L.gpu_v7b_snap_launch)(C.byref(sa)), "snapshot entry")
    torch.cuda.synchronize()
    snap = devbuf.cpu().numpy().copy()
    common = (B, G, Cp, plan["ncls"], q, d["nodes"].data_ptr(), d["block_v0"].data_ptr(), d["block_v1"].data_ptr(),
              d["fac_start"].data_ptr(), d["g2row"].data_ptr(), d["ms_off"].data_ptr(), d["ms_cls"].data_ptr(),
              d["ms_base"].data_ptr(), d["ms_dev"].data_ptr(), devbuf.data_ptr(), d["need_off"].data_ptr(),
              d["qlb"].data_ptr(), d["qhb"].data_ptr(), lvals.data_ptr(), dV.data_ptr())
    ca = GpuV7CombineArgs(S - 1, q, Cp, d["qlb"].data_ptr(), d["qhb"].data_ptr(), carry.data_ptr(),
                          d["bidx"].data_ptr(), lvals.data_ptr(), answers.data_ptr())
    if session:
        fen = torch.empty(B * Cp, dtype=torch.int64, device=dev)
        leaf = torch.empty(B * Cp, dtype=torch.int64, device=dev)
        ra = GpuSessRunArgs(*common, fen.data_ptr(), leaf.data_ptr(), 256)
        snap_dev = devbuf.clone()   # each batch replays from the snapshots (panel_gpu_session.cpp:111-131)
        for _ in range(max(1, batches)):
            devbuf.copy_(snap_dev)
            _check(L.gpu_sess_reset_launch(C.byref(GpuSessResetArgs(B, Cp, fen.data_ptr(), leaf.data_ptr()))),
                   "gpu_sess_reset_launch")
            _check(L.gpu_sess_run_launch(C.byref(ra)), "gpu_sess_run_launch")
            _check(L.bw_v7_carry_launch(B, Cp, d["vbase"].data_ptr(), dV.data_ptr(), carry.data_ptr(), None),
                   "bw_v7_carry_launch")
            _check(L.gpu_sess_combine_launch(C.byref(ca)), "gpu_sess_combine_launch")
    else:
        _check(L.gpu_v7b_launch(C.byref(GpuV7bArgs(*common, 256, 0))), "gpu_v7b_launch")
        _check(L.bw_v7_carry_launch(B, Cp, d["vbase"].data_ptr(), dV.data_ptr(), carry.data_ptr(), None),
               "bw_v7_carry_launch")
        _check(L.gpu_v7b_combine_launch(C.byref(ca)), "gpu_v7b_combine_launch")
    torch.cuda.synchronize()
    return answers.cpu().numpy(), snap


def replay_noalloc(parent, n_keys: int, events, queries, *, blocks: int = 0, chain: bool = False):
    """The replay through bw_replay_launch_noalloc: for callers that cannot allocate
    device memory when they run it, the scratch comes from the library's fixed
    region instead of a workspace.  Only the answer buffer is created here (by the
    caller's side, as any output); the native call allocates nothing.  Workloads
    whose scratch exceeds the region raise ValueError."""
    torch = _torch()
    L = gpu_lib()
    L.bw_replay_launch_noalloc.argtypes = [C.POINTER(BwReplayArgs), C.POINTER(C.c_int32)]
    a = BwReplayArgs()
    a.n_states, a.n_keys = int(parent.numel()), int(n_keys)
    a.n_events, a.n_queries = int(events.shape[0]), int(queries.shape[0])
    a.blocks, a.flags = int(blocks), BW_REPLAY_CHAIN_HINT if chain else 0
    answers = torch.empty(a.n_queries, dtype=torch.int64, device=parent.device)
    a.parent = parent.data_ptr()
    a.events = events.data_ptr() if a.n_events else None
    a.queries = queries.data_ptr() if a.n_queries else None
    a.answers = answers.data_ptr() if a.n_queries else None
    a.stream = torch.cuda.current_stream(parent.device).cuda_stream
    st = C.c_int32(0)
    rc = L.bw_replay_launch_noalloc(C.byref(a), C.byref(st))
    if rc == BW_EINVAL:
        raise ValueError("bw_replay_launch_noalloc rejected the call (see stderr)")
    _check(rc, "bw_replay_launch_noalloc")
    if st.value:
        raise ValueError(f"replay input rejected on the device: {STATUS_NAMES.get(st.value, st.value)}")
    return answers


class CsrIndex:
    """Sparse-key CSR rank-LUT on the device (CsrBase of sparse_engine.hpp:70-102 over
    a u64 key universe [0, 2^key_bits)).  Built from (key, amount) pairs by
    bw_csr_build; the index lives in a workspace held by this object.

    point(keys) -> rank where present, -rank-1 where absent (rank = keys below);
    range(bounds (n, 2)) -> (n, 2) int64 (rank(hi) - rank(lo), amount sum over [lo, hi))."""

    def __init__(self, keys, amounts, *, key_bits: int = 40, lut_budget_bytes: int = 64 << 20):
        torch = _torch()
        L = gpu_lib()
        n = int(keys.numel())
        assert keys.is_cuda and amounts.is_cuda and amounts.numel() == n
        self.device = keys.device
        nbytes = C.c_size_t(0)
        _check(L.bw_csr_workspace_size(n, int(key_bits), int(lut_budget_bytes), C.byref(nbytes)),
               "bw_csr_workspace_size")
        self.workspace = torch.empty(max(256, nbytes.value), dtype=torch.uint8, device=self.device)
        self.idx = BwCsr()
        st = torch.cuda.current_stream(self.device).cuda_stream
        _check(L.bw_csr_build(keys.contiguous().data_ptr() if n else None,
                              amounts.contiguous().data_ptr() if n else None, n, int(key_bits),
                              int(lut_budget_bytes), self.workspace.data_ptr(), self.workspace.numel(), st,
                              C.byref(self.idx)), "bw_csr_build")
        self.key_bits, self.shift, self.n_buckets = key_bits, self.idx.shift, self.idx.n_buckets
        self.lut_bytes = self.n_buckets * 4
        self._src = (keys, amounts, n, int(lut_budget_bytes))

    def rebuild(self):
        """Enqueue the build again into the same workspace (timing, refresh)."""
        torch = _torch()
        keys, amounts, n, budget = self._src
        st = torch.cuda.current_stream(self.device).cuda_stream
        _check(gpu_lib().bw_csr_build(keys.data_ptr() if n else None, amounts.data_ptr() if n else None, n,
                                      int(self.key_bits), budget, self.workspace.data_ptr(),
                                      self.workspace.numel(), st, C.byref(self.idx)), "bw_csr_build")

    def status(self) -> int:
        """0, or 1 when a build key lay outside [0, 2^key_bits) (synchronises)."""
        st = C.c_int32(0)
        _check(gpu_lib().bw_csr_status(C.byref(self.idx), C.byref(st)), "bw_csr_status")
        return int(st.value)

    def count(self) -> int:
        torch = _torch()
        c = torch.empty(1, dtype=torch.int64, device=self.device)
        c.copy_(self._view(self.idx.count, 1, torch.int64))
        return int(c.item())

    def _view(self, ptr: int, n: int, dtype):
        torch = _torch()
        base = self.workspace.data_ptr()
        esz = torch.tensor([], dtype=dtype).element_size()
        off = (ptr - base)
        return self.workspace[off:off + n * esz].view(dtype)

    def arrays(self):
        """(keys u64 as int64, pre int64) device views of the built index."""
        torch = _torch()
        m = self.count()
        return self._view(self.idx.keys, m, torch.int64), self._view(self.idx.pre, m, torch.int64)

    def point(self, keys, out=None):
        torch = _torch()
        n = int(keys.numel())
        out = torch.empty(n, dtype=torch.int64, device=self.device) if out is None else out
        st = torch.cuda.current_stream(self.device).cuda_stream
        _check(gpu_lib().bw_csr_point(C.byref(self.idx), keys.data_ptr() if n else None, n,
                                      out.data_ptr() if n else None, st), "bw_csr_point")
        return out

    def range(self, bounds, out=None):
        torch = _torch()
        n = int(bounds.numel()) // 2
        out = torch.empty((n, 2), dtype=torch.int64, device=self.device) if out is None else out
        st = torch.cuda.current_stream(self.device).cuda_stream
        _check(gpu_lib().bw_csr_range(C.byref(self.idx), bounds.data_ptr() if n else None, n,
                                      out.data_ptr() if n else None, st), "bw_csr_range")
        return out

    def events(self, states, keys, deltas):
        """Event records over the index's ranks (bw_csr_events): an (n, 2) int64 tensor
        of {u32 state, u32 rank, i64 delta}; states u32-valued int32, keys u64 as int64."""
        torch = _torch()
        L = gpu_lib()
        L.bw_csr_events.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                    C.c_void_p]
        n = int(keys.numel())
        out = torch.empty((max(n, 1), 2), dtype=torch.int64, device=self.device)[:n]
        st = torch.cuda.current_stream(self.device).cuda_stream
        _check(L.bw_csr_events(C.byref(self.idx), states.data_ptr() if n else None, keys.data_ptr() if n else None,
                               deltas.data_ptr() if n else None, n, out.data_ptr() if n else None, st),
               "bw_csr_events")
        return out

    def queries(self, states, lo, hi=None):
        """Query records over rank intervals (bw_csr_queries): point lookups of lo
        (hi None) or range lookups over keys [lo, hi); an (n, 3) int32 tensor."""
        torch = _torch()
        L = gpu_lib()
        L.bw_csr_queries.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                     C.c_void_p]
        n = int(lo.numel())
        out = torch.empty((max(n, 1), 3), dtype=torch.int32, device=self.device)[:n]
        st = torch.cuda.current_stream(self.device).cuda_stream
        _check(L.bw_csr_queries(C.byref(self.idx), states.data_ptr() if n else None, lo.data_ptr() if n else None,
                                hi.data_ptr() if (n and hi is not None) else None, n,
                                out.data_ptr() if n else None, st), "bw_csr_queries")
        return out
