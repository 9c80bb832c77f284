"""cs_solve_cg_noalloc: the CG solve for callers that cannot allocate device
memory (an engine that owns every device allocation, a real-time loop that must
not enter the CUDA allocator).  The caller hands over the block system already
in device memory; the entry point keeps its work vectors in a fixed device
array instead of allocating.  Checked through the C ABI against the context's
cs_solve_cg and the oracle's Solve_CG on the same system, on two calls in a
row, within the parity tolerance of the other GPU tests (RTOL relative), and on
a solve cut off by its iteration cap, where the reference reports the tolerance
and the cap (matrix_square_sparse.cpp:338-406)."""
import ctypes
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-9
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_noalloc_cg_matches_context_solve():
    import torch

    from cloth_sim_self_collision_gb300 import _native as N
    from cloth_sim_self_collision_gb300 import build, scene
    from cloth_sim_self_collision_gb300.context import ClothContext
    from oracle import oracle as O

    build.build()
    O.build("port")
    L = N.load()
    torch.cuda.set_device(0)
    c = scene.config_small()
    arr = dict(np.load(os.path.join(GOLDEN, "small_21.npz")))
    ctx = ClothContext(0)
    cid = ctx.add_cloth(c)
    vd, vc, b = ctx.assemble(cid, arr["probe_x"], arr["probe_v"])
    rp, ci = ctx.pattern(cid)
    x_ref, conv_ref, it_ref = ctx.cg(cid, b, 1e-6, 1000)
    orc = O.OracleCloth(O.OracleLib("port"), c)
    vdo, vco, bo = orc.assemble(arr["probe_x"], arr["probe_v"])
    assert np.array_equal(vdo, vd) and np.array_equal(vco, vc) and np.array_equal(bo, b)
    x_orc, conv_orc, it_orc = orc.cg(b, 1e-6, 1000)
    x_cut, conv_cut, it_cut = orc.cg(b, 1e-6, 5)
    assert conv_cut == 1e-6 and it_cut == 5

    dev = torch.device("cuda", 0)
    t_rp = torch.from_numpy(rp.astype(np.int32)).to(dev)
    t_ci = torch.from_numpy(ci.astype(np.int32)).to(dev)
    t_vc = torch.from_numpy(vc).to(dev)
    t_vd = torch.from_numpy(vd).to(dev)
    t_b = torch.from_numpy(b).to(dev)
    t_x = torch.full_like(t_b, float("nan"))
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize()
    for call in range(2):
        conv = ctypes.c_double()
        it = ctypes.c_int()
        rc = L.cs_solve_cg_noalloc(t_rp.data_ptr(), t_ci.data_ptr(), t_vc.data_ptr(), t_vd.data_ptr(),
                                   t_b.data_ptr(), t_x.data_ptr(), c.np, 1e-6, 1000, ctypes.byref(conv),
                                   ctypes.byref(it), ctypes.c_void_p(stream))
        assert rc == N.CS_OK, (call, rc)
        x = t_x.cpu().numpy()
        scale = max(1.0, np.abs(x_ref).max())
        assert np.abs(x - x_ref).max() <= RTOL * scale, (call, np.abs(x - x_ref).max())
        assert abs(it.value - it_ref) <= 1, (call, it.value, it_ref)
        assert abs(conv.value - conv_ref) <= 1e-6 * conv_ref + 1e-300, (call, conv.value, conv_ref)
        scale = max(1.0, np.abs(x_orc).max())
        assert np.abs(x - x_orc).max() <= RTOL * scale, (call, np.abs(x - x_orc).max())
        assert abs(it.value - it_orc) <= 1, (call, it.value, it_orc)
        assert abs(conv.value - conv_orc) <= 1e-6 * conv_orc + 1e-300, (call, conv.value, conv_orc)
    # a solve stopped by its cap: conv and iter keep the tolerance and the cap
    for call in range(2):
        conv = ctypes.c_double()
        it = ctypes.c_int()
        rc = L.cs_solve_cg_noalloc(t_rp.data_ptr(), t_ci.data_ptr(), t_vc.data_ptr(), t_vd.data_ptr(),
                                   t_b.data_ptr(), t_x.data_ptr(), c.np, 1e-6, 5, ctypes.byref(conv),
                                   ctypes.byref(it), ctypes.c_void_p(stream))
        assert rc == N.CS_OK, (call, rc)
        assert conv.value == 1e-6 and it.value == 5, (call, conv.value, it.value)
        x = t_x.cpu().numpy()
        assert np.abs(x - x_cut).max() <= RTOL * max(1.0, np.abs(x_cut).max()), (call, np.abs(x - x_cut).max())
    orc.close()
    ctx.close()


def test_noalloc_rejects_oversized_systems():
    from cloth_sim_self_collision_gb300 import _native as N
    from cloth_sim_self_collision_gb300 import build

    build.build()
    L = N.load()
    dummy = ctypes.c_void_p(16)
    conv = ctypes.c_double()
    it = ctypes.c_int()
    rc = L.cs_solve_cg_noalloc(dummy, dummy, dummy, dummy, dummy, dummy, 16385, 1e-6, 10, ctypes.byref(conv),
                               ctypes.byref(it), None)
    assert rc == N.CS_ERR_CAPACITY
