"""The allocation-free replay entry point (bw_replay_launch_noalloc).

Hosts that cannot allocate device memory when they run a replay (a plugin with a
fixed memory budget, a loop that must not block in the allocator) call this entry
point; its scratch is a fixed region inside the library.  These tests call it
through the C ABI twice in a row on different workloads and require the answers to
equal, bit for bit, those of the workspace-based bw_replay_launch on the same
inputs and, on one more workload, to the oracle's; they check that repeated calls
leave the device's free memory unchanged, and that an oversized workload and a
caller-supplied workspace are refused with an error instead of running.  The file is named to be collected
last, so a run that stops at the first failure has already run every other test."""
from __future__ import annotations

import numpy as np
import pytest

import evgen

pytestmark = pytest.mark.gpu


def _case(seed, kind, S, C, E, Q):
    rng = np.random.default_rng(seed)
    return (evgen.make_tree(S, kind, rng), C, evgen.make_events(S, C, E, rng, zipf=1.1),
            evgen.make_queries(S, C, Q, rng))


def test_noalloc_matches_workspace_path_twice(bw, torch_cuda):
    cases = [_case(21, "fork", 6000, 4096, 150000, 80000), _case(22, "chain", 3000, 20000, 90000, 60000)]
    for parent, C, ev, qs in cases:   # two calls in a row: the region is reused
        p, e, q = evgen.to_device(torch_cuda, parent, ev, qs)
        got = bw.replay_noalloc(p, C, e, q).cpu().numpy()
        want = bw.replay(p, C, e, q).cpu().numpy()
        np.testing.assert_array_equal(got, want)


def test_noalloc_matches_oracle_and_allocates_nothing(bw, torch_cuda, oracle_mod):
    import ctypes as C_
    parent, C, ev, qs = _case(25, "fork", 4000, 3000, 100000, 60000)
    p, e, q = evgen.to_device(torch_cuda, parent, ev, qs)
    L = bw.gpu_lib()
    L.bw_replay_launch_noalloc.argtypes = [C_.POINTER(bw.BwReplayArgs), C_.POINTER(C_.c_int32)]
    answers = torch_cuda.empty(len(qs), dtype=torch_cuda.int64, device=p.device)
    a = bw.BwReplayArgs()
    a.n_states, a.n_keys, a.n_events, a.n_queries = len(parent), C, len(ev), len(qs)
    a.parent, a.events, a.queries, a.answers = p.data_ptr(), e.data_ptr(), q.data_ptr(), answers.data_ptr()
    a.stream = torch_cuda.cuda.current_stream(p.device).cuda_stream
    st = C_.c_int32(-1)
    assert L.bw_replay_launch_noalloc(C_.byref(a), C_.byref(st)) == 0 and st.value == 0   # warm-up call
    torch_cuda.cuda.synchronize()
    free0, _ = torch_cuda.cuda.mem_get_info()
    for _ in range(3):
        assert L.bw_replay_launch_noalloc(C_.byref(a), C_.byref(st)) == 0 and st.value == 0
    torch_cuda.cuda.synchronize()
    free1, _ = torch_cuda.cuda.mem_get_info()
    assert free1 == free0, "the allocation-free entry changed the device's free memory"
    np.testing.assert_array_equal(answers.cpu().numpy(), oracle_mod.ev_sweep(parent, C, ev, qs))


def test_noalloc_rejects_oversized_workload(bw, torch_cuda):
    # a key domain whose dense carry rows alone exceed the fixed region
    parent, C, ev, qs = _case(23, "chain", 200, 1 << 24, 2000, 500)
    p, e, q = evgen.to_device(torch_cuda, parent, ev, qs)
    with pytest.raises(ValueError, match="rejected the call"):
        bw.replay_noalloc(p, C, e, q, blocks=4)
    # the context stays usable
    parent, C, ev, qs = _case(24, "fork", 500, 256, 5000, 2000)
    p, e, q = evgen.to_device(torch_cuda, parent, ev, qs)
    np.testing.assert_array_equal(bw.replay_noalloc(p, C, e, q).cpu().numpy(),
                                  bw.replay(p, C, e, q).cpu().numpy())


def test_noalloc_refuses_caller_workspace(bw, torch_cuda):
    import ctypes as C
    L = bw.gpu_lib()
    L.bw_replay_launch_noalloc.argtypes = [C.POINTER(bw.BwReplayArgs), C.POINTER(C.c_int32)]
    a = bw.BwReplayArgs()
    a.n_states, a.n_keys, a.workspace_bytes = 1, 1, 256
    assert L.bw_replay_launch_noalloc(C.byref(a), None) == bw.BW_EINVAL
