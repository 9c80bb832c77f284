"""The C-ABI library loads and exports every symbol include/clothgpu.h declares
(no compute call: runs without a GPU)."""
import ctypes
import os
import re

from cloth_sim_self_collision_gb300 import _native as N
from cloth_sim_self_collision_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "clothgpu.h")).read()
    return sorted(set(re.findall(r"\b(cs_[a-z0-9_]+)\s*\(", src)))


def test_header_matches_binding_list():
    assert declared() == sorted(N.EXPORTS)


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(build.build())
    for name in declared():
        assert hasattr(lib, name), name


def test_no_device_is_reported_not_crashed():
    import torch
    if torch.cuda.is_available():
        return
    L = N.load(build.build())
    h = ctypes.c_void_p()
    assert L.cs_create(0, N.CS_PREC_FP64, ctypes.byref(h)) == N.CS_ERR_NO_DEVICE
