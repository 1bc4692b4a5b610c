"""CPU checks of the C ABI: the CUDA library builds for sm_103a, loads without a
GPU, and exports every function include/*.h declares; struct layouts match the
reference's gpu_v7.h sizes."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_functions(header: Path):
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    names = re.findall(r"^\s*(?:int|void|size_t|uint64_t|int64_t|int32_t|const char\s*\*)\s+(\w+)\s*\(",
                       text, flags=re.M)
    return sorted(set(names))


def test_gpu_library_exports_header(bw):
    bw.build()
    lib = C.CDLL(str(bw._build.GPU_LIB))
    names = declared_functions(ROOT / "include" / "bw_gpu.h")
    assert "bw_replay_launch" in names and "gpu_v7_launch" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_sizes(bw):
    class GpuV7Node(C.Structure):
        _fields_ = [("kind", C.c_int32), ("g_old", C.c_int32), ("c_old", C.c_int32),
                    ("ti_old", C.c_int32), ("g_new", C.c_int32), ("c_new", C.c_int32),
                    ("ti_new", C.c_int32), ("amt_old", C.c_int64), ("amt_new", C.c_int64),
                    ("fac_val", C.c_int64), ("fac_prev", C.c_int64), ("ex_old", C.c_uint8),
                    ("ex_new", C.c_uint8), ("pad", C.c_uint8 * 6)]
    assert C.sizeof(GpuV7Node) == 72
    assert C.sizeof(bw.BwReplayArgs) == 96  # matches the C layout with natural padding


def test_no_gpu_path_raises_without_cuda(bw):
    import torch
    if torch.cuda.is_available():
        return
    import pytest
    with pytest.raises(RuntimeError):
        bw.replay(torch.zeros(1, dtype=torch.int32), 1, torch.zeros((0, 2), dtype=torch.int64),
                  torch.zeros((0, 3), dtype=torch.int32))
