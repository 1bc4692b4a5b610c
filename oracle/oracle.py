"""ctypes wrapper around liboracle.so -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this module.  It exposes the CPU restatements in bw_oracle.c:

* ``fixture_*`` / ``workload_*`` / ``direct_scan``: the reference-native semantics
  (common.hpp:112-155 loader, common.hpp:279-374 make_workload, oracle.cpp:213-451
  direct-scan oracle);
* ``ev_bruteforce`` / ``ev_sweep`` / ``ev_blocks``: the event-model checkers
  (ancestor walk, batch_engine_v7.hpp:1021-1059 preorder replay,
  batch_engine_v7.hpp:832-968 block-parallel chain executor).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"

EVENT_DTYPE = np.dtype([("state", "<u4"), ("key", "<u4"), ("delta", "<i8")])
QUERY_DTYPE = np.dtype([("state", "<u4"), ("lo", "<u4"), ("hi", "<u4")])


def build(force: bool = False) -> Path:
    """Compile liboracle.so in place (gcc, a few seconds)."""
    src = HERE / "bw_oracle.c"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    return LIB_PATH


class _Fixture(C.Structure):
    _fields_ = [("n", C.c_int64), ("groups", C.c_int32), ("unit", C.c_int32),
                ("t_min", C.c_int64), ("t_max", C.c_int64), ("row_t", C.c_void_p),
                ("rows", C.c_void_p), ("factor", C.c_void_p), ("labels", C.c_void_p)]


class _Workload(C.Structure):
    _fields_ = [("n_states", C.c_int32), ("topology", C.c_int32), ("seed", C.c_int32),
                ("factor_period", C.c_int32), ("q", C.c_int32), ("per_state", C.c_int32),
                ("factor_pct", C.c_int32), ("n_base", C.c_int64), ("groups", C.c_int32),
                ("n_inserted", C.c_int32), ("t_min", C.c_int64), ("t_max", C.c_int64),
                ("parent", C.c_void_p), ("op", C.c_void_p), ("eg", C.c_void_p),
                ("eid", C.c_void_p), ("eval", C.c_void_p), ("et", C.c_void_p),
                ("qlo", C.c_void_p), ("qhi", C.c_void_p), ("ins_t", C.c_void_p),
                ("ins_g", C.c_void_p), ("endpoints", C.c_void_p), ("n_endpoints", C.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        L.bwo_sha256_hex.argtypes = [C.c_void_p, C.c_size_t, C.c_char_p]
        L.bwo_fnv1a.argtypes = [C.c_void_p, C.c_size_t]
        L.bwo_fnv1a.restype = C.c_uint64
        L.bwo_fixture_parse.argtypes = [C.c_void_p, C.c_size_t, C.POINTER(_Fixture)]
        L.bwo_workload_make.argtypes = [C.POINTER(_Fixture)] + [C.c_int32] * 7 + [C.POINTER(_Workload)]
        L.bwo_workload_free.argtypes = [C.POINTER(_Workload)]
        L.bwo_direct_scan.argtypes = [C.POINTER(_Fixture), C.POINTER(_Workload), C.c_void_p]
        ev_args = [C.c_int32, C.c_void_p, C.c_uint32, C.c_int64, C.c_void_p, C.c_int64,
                   C.c_void_p, C.c_void_p]
        L.bwo_ev_bruteforce.argtypes = [C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                        C.c_void_p, C.c_void_p]
        L.bwo_ev_sweep.argtypes = ev_args
        L.bwo_ev_sweep_prefix.argtypes = ev_args + [C.c_int64, C.POINTER(C.c_int64),
                                                    C.POINTER(C.c_double)]
        L.bwo_ev_blocks.argtypes = ev_args + [C.c_int32, C.c_int32]
        L.bwo_max_threads.restype = C.c_int
        L.bwo_csr_build.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                    C.POINTER(C.c_int64)]
        L.bwo_csr_point.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]
        L.bwo_csr_range.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def sha256_hex(buf) -> str:
    a = np.ascontiguousarray(np.frombuffer(memoryview(buf).cast("B"), dtype=np.uint8))
    out = C.create_string_buffer(65)
    lib().bwo_sha256_hex(_ptr(a) if a.size else None, a.size, out)
    return out.value.decode()


def fnv1a(buf) -> int:
    a = np.ascontiguousarray(np.frombuffer(memoryview(buf).cast("B"), dtype=np.uint8))
    return int(lib().bwo_fnv1a(_ptr(a) if a.size else None, a.size))


class Fixture:
    """A parsed BWBASE02 image (keeps the bytes alive)."""

    def __init__(self, image: bytes):
        self.image = np.frombuffer(image, dtype=np.uint8).copy()
        self.s = _Fixture()
        rc = lib().bwo_fixture_parse(_ptr(self.image), self.image.size, C.byref(self.s))
        if rc:
            raise ValueError(f"malformed BWBASE02 fixture (rc={rc})")


def direct_scan(fx: Fixture, n_states: int, topology: int, seed: int, factor_period: int,
                q: int, per_state: bool = True, factor_pct: int = -1) -> np.ndarray:
    """Answers of the independent direct-scan oracle, order v=1..S-1, k=0..q-1."""
    w = _Workload()
    rc = lib().bwo_workload_make(C.byref(fx.s), n_states, topology, seed, factor_period, q,
                                 int(per_state), factor_pct, C.byref(w))
    if rc:
        raise ValueError(f"workload rejected (rc={rc})")
    try:
        ans = np.zeros((n_states - 1) * q, dtype=np.int64)
        rc = lib().bwo_direct_scan(C.byref(fx.s), C.byref(w), _ptr(ans))
        if rc == 6:
            raise OverflowError("an exact answer does not fit int64")
        if rc:
            raise RuntimeError(f"direct scan failed rc={rc}")
        return ans
    finally:
        lib().bwo_workload_free(C.byref(w))


def direct_scan_declared(fx: Fixture, decl) -> np.ndarray:
    """Direct-scan oracle answers of an explicit declared workload: ``decl`` has
    n-state arrays parent/op/g/id/val/t, ranges qlo/qhi (n_states*q per state or q
    shared), ins_t/ins_g of the inserted rows, q and per_state (the reference fuzz's
    Workload, fuzz_fullpath.cpp:196-283)."""
    S, q = int(decl.parent.size), int(decl.q)
    keep = {
        "parent": np.ascontiguousarray(decl.parent, np.int32), "op": np.ascontiguousarray(decl.op, np.uint8),
        "eg": np.ascontiguousarray(decl.g, np.int32), "eid": np.ascontiguousarray(decl.id, np.int64),
        "eval": np.ascontiguousarray(decl.val, np.int64), "et": np.ascontiguousarray(decl.t, np.int64),
        "qlo": np.ascontiguousarray(decl.qlo, np.int64), "qhi": np.ascontiguousarray(decl.qhi, np.int64),
        "ins_t": np.ascontiguousarray(decl.ins_t, np.int64).reshape(-1),
        "ins_g": np.ascontiguousarray(decl.ins_g, np.int32).reshape(-1)}
    w = _Workload()
    w.n_states, w.q, w.per_state = S, q, int(bool(decl.per_state))
    w.n_base, w.groups, w.n_inserted = fx.s.n, fx.s.groups, int(keep["ins_t"].size)
    w.t_min, w.t_max = fx.s.t_min, fx.s.t_max
    for k, a in keep.items():
        setattr(w, k, _ptr(a) if a.size else None)
    ans = np.zeros((S - 1) * q, dtype=np.int64)
    rc = lib().bwo_direct_scan(C.byref(fx.s), C.byref(w), _ptr(ans))
    if rc == 6:
        raise OverflowError("an exact answer does not fit int64")
    if rc:
        raise RuntimeError(f"direct scan failed rc={rc}")
    return ans


STREAM_DTYPE = np.dtype([("kind", "<u4"), ("state", "<u4"), ("qidx", "<u4"), ("g", "<i4"), ("w", "<i4"),
                         ("a", "<i8"), ("b", "<i8")])   # 36 bytes, packed


def stream_answers(fixture: bytes, stream: bytes) -> np.ndarray:
    """The reference's answers for a BWLEV001 event stream (emit_events.cpp:5-8,
    21-27): replay the records in order over the fixture's base rows, answer each
    query as the sum over groups of factor x the live amounts with t in [lo, hi)
    (external/dd_probe/src/main.rs:66-80), and order the answers by (state, qidx)
    without state 0 (main.rs:245-262).  Wrapping int64 throughout.  A direct
    restatement over per-group live-mass arrays: Python loops, test sizes only."""
    import struct
    assert stream[:8] == b"BWLEV001"
    (n,) = struct.unpack_from("<Q", stream, 8)
    assert len(stream) == 16 + 36 * n
    rec = np.frombuffer(stream, dtype=STREAM_DTYPE, count=n, offset=16)
    rows, groups = struct.unpack_from("<qi", fixture, 8)
    base = np.frombuffer(fixture, dtype=np.dtype([("t", "<i8"), ("a", "<i8"), ("g", "<i4"), ("p", "<i4")]),
                         count=rows, offset=64)
    mul = [int(x) for x in np.frombuffer(fixture, dtype="<i8", count=groups, offset=64 + 24 * rows)]
    times = np.unique(np.concatenate([base["t"], rec["a"][rec["kind"] == 0]]))
    live = np.zeros((groups, times.size), dtype=np.int64)
    np.add.at(live, (base["g"], np.searchsorted(times, base["t"])), base["a"])
    M = (1 << 64) - 1
    out = []
    with np.errstate(over="ignore"):
        for r in rec:
            k = int(r["kind"])
            if k == 0:
                live[r["g"], np.searchsorted(times, r["a"])] += np.int64(r["w"]) * r["b"]
            elif k == 1:
                mul[int(r["g"])] = int(r["a"])
            else:
                lo, hi = np.searchsorted(times, [r["a"], r["b"]])
                ans = 0
                for g in range(groups):
                    ans += mul[g] * int(live[g, lo:hi].sum()) if hi > lo else 0
                ans &= M
                out.append((int(r["state"]), int(r["qidx"]), ans - (1 << 64) if ans >> 63 else ans))
    out.sort()
    return np.array([a for s, _, a in out if s != 0], dtype=np.int64)


def _ev_arrays(parent, events, queries):
    parent = np.ascontiguousarray(parent, dtype=np.int32)
    events = np.ascontiguousarray(events, dtype=EVENT_DTYPE)
    queries = np.ascontiguousarray(queries, dtype=QUERY_DTYPE)
    return parent, events, queries


def ev_bruteforce(parent, events, queries) -> np.ndarray:
    parent, events, queries = _ev_arrays(parent, events, queries)
    ans = np.zeros(len(queries), dtype=np.int64)
    rc = lib().bwo_ev_bruteforce(len(parent), _ptr(parent), len(events), _ptr(events),
                                 len(queries), _ptr(queries), _ptr(ans))
    if rc not in (0, 6):
        raise ValueError(f"bad event-model input (rc={rc})")
    return ans


def ev_sweep(parent, n_keys: int, events, queries) -> np.ndarray:
    parent, events, queries = _ev_arrays(parent, events, queries)
    ans = np.zeros(len(queries), dtype=np.int64)
    rc = lib().bwo_ev_sweep(len(parent), _ptr(parent), n_keys, len(events), _ptr(events),
                            len(queries), _ptr(queries), _ptr(ans))
    if rc:
        raise ValueError(f"bad event-model input (rc={rc})")
    return ans


def ev_forest(state_off, event_off, query_off, n_keys, parent, events, queries, fn=None) -> np.ndarray:
    """Answers of a forest of independent trees: each tree's slice replayed alone
    with the preorder checker (or ``fn``), concatenated in tree order."""
    fn = fn or (lambda p, C, e, q: ev_sweep(p, C, e, q))
    out = np.zeros(int(query_off[-1]), dtype=np.int64)
    for t in range(len(n_keys)):
        s0, s1 = int(state_off[t]), int(state_off[t + 1])
        e0, e1 = int(event_off[t]), int(event_off[t + 1])
        q0, q1 = int(query_off[t]), int(query_off[t + 1])
        if q1 > q0:
            out[q0:q1] = fn(parent[s0:s1], int(n_keys[t]), events[e0:e1], queries[q0:q1])
    return out


def ev_sweep_prefix(parent, n_keys: int, events, queries, limit_steps: int):
    """Preorder replay of the first `limit_steps` states; returns (answers,
    answered, seconds of the replay loop)."""
    parent, events, queries = _ev_arrays(parent, events, queries)
    ans = np.zeros(len(queries), dtype=np.int64)
    done = C.c_int64(0)
    secs = C.c_double(0.0)
    rc = lib().bwo_ev_sweep_prefix(len(parent), _ptr(parent), n_keys, len(events), _ptr(events),
                                   len(queries), _ptr(queries), _ptr(ans), limit_steps,
                                   C.byref(done), C.byref(secs))
    if rc:
        raise ValueError(f"bad event-model input (rc={rc})")
    return ans, int(done.value), float(secs.value)


def ev_blocks(parent, n_keys: int, events, queries, blocks: int = 0, threads: int = 0) -> np.ndarray:
    parent, events, queries = _ev_arrays(parent, events, queries)
    ans = np.zeros(len(queries), dtype=np.int64)
    rc = lib().bwo_ev_blocks(len(parent), _ptr(parent), n_keys, len(events), _ptr(events),
                             len(queries), _ptr(queries), _ptr(ans), blocks, threads)
    if rc:
        raise ValueError(f"block executor needs a chain and valid input (rc={rc})")
    return ans


def csr_build(keys, amounts):
    """Sorted distinct keys and their cumulative amount prefix (build_csr_base)."""
    k = np.ascontiguousarray(keys, dtype=np.uint64)
    a = np.ascontiguousarray(amounts, dtype=np.int64)
    assert k.shape == a.shape
    uk = np.empty(max(1, k.size), np.uint64)
    pre = np.empty(max(1, k.size), np.int64)
    m = C.c_int64(0)
    rc = lib().bwo_csr_build(_ptr(k), _ptr(a), k.size, _ptr(uk), _ptr(pre), C.byref(m))
    if rc:
        raise MemoryError("bwo_csr_build")
    return uk[:m.value].copy(), pre[:m.value].copy()


def csr_point(ukeys, q):
    uk = np.ascontiguousarray(ukeys, dtype=np.uint64)
    qq = np.ascontiguousarray(q, dtype=np.uint64)
    out = np.empty(qq.size, np.int64)
    lib().bwo_csr_point(_ptr(uk), uk.size, _ptr(qq), qq.size, _ptr(out))
    return out


def csr_range(ukeys, pre, bounds):
    """bounds: (n, 2) u64 [lo, hi) pairs -> (n, 2) int64 (count, amount sum)."""
    uk = np.ascontiguousarray(ukeys, dtype=np.uint64)
    pr = np.ascontiguousarray(pre, dtype=np.int64)
    b = np.ascontiguousarray(bounds, dtype=np.uint64).reshape(-1, 2)
    out = np.empty((b.shape[0], 2), np.int64)
    lib().bwo_csr_range(_ptr(uk), _ptr(pr), uk.size, _ptr(b), b.shape[0], _ptr(out))
    return out


def max_threads() -> int:
    return int(lib().bwo_max_threads())


def reference_dir() -> Path | None:
    """The reference checkout used to build the pinning binaries: $BW_REFERENCE_DIR,
    else a ``reference`` directory beside this repository; None when neither holds
    the reference sources."""
    cand = [os.environ.get("BW_REFERENCE_DIR"), str(HERE.parent.parent / "reference")]
    for c in cand:
        if c and (Path(c) / "src" / "oracle.cpp").exists():
            return Path(c)
    return None


def ref_binary(name: str, states: int) -> Path | None:
    """Path of a reference binary built by oracle/ref.mk, when present."""
    p = HERE / "_ref" / f"{name}_{states}"
    return p if p.exists() and os.access(p, os.X_OK) else None
