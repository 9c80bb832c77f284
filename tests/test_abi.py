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


def test_server_without_device_is_reported_not_crashed():
    import torch
    if torch.cuda.is_available():
        return
    L = N.load(build.build())
    h = ctypes.c_void_p()
    cfg = N.CsServerConfig(0, N.CS_PREC_MIXED, 1e9, 0)
    assert L.cs_server_create(ctypes.byref(cfg), ctypes.byref(h)) == N.CS_ERR_NO_DEVICE
    bad = N.CsServerConfig(0, N.CS_PREC_MIXED, 0.0, 0)
    assert L.cs_server_create(ctypes.byref(bad), ctypes.byref(h)) == N.CS_ERR_ARG


def test_scene_estimate_runs_on_the_host():
    """The admission estimate needs no device and grows with the scene."""
    from cloth_sim_self_collision_gb300 import scene
    from cloth_sim_self_collision_gb300.serve import scene_device_bytes
    small = scene_device_bytes(scene.square_cloth(11, 1.0, 0.5))
    big = scene_device_bytes(scene.square_cloth(41, 1.0, 0.5))
    assert 0 < small < big
    assert 1.5e3 * 41 * 41 < big < 2e4 * 41 * 41  # a few KB per vertex
