"""The library's host-side topology builder (no GPU needed) against the
reference's BVH and matrix pattern: golden fixtures and the oracle."""
import ctypes
import json
import os

import numpy as np
import pytest

from cloth_sim_self_collision_gb300 import _native as N
from cloth_sim_self_collision_gb300 import build, scene
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def lib():
    return N.load(build.build())


def bvh(L, c):
    X = np.ascontiguousarray(c.X0)
    tri = np.ascontiguousarray(c.tri)
    nn = ctypes.c_int()
    assert L.cs_build_bvh(c.np, N.dp(X), c.nt, N.ip(tri), None, 0, ctypes.byref(nn)) == N.CS_OK
    out = np.zeros(3 * nn.value, np.int32)
    assert L.cs_build_bvh(c.np, N.dp(X), c.nt, N.ip(tri), N.ip(out), out.size, ctypes.byref(nn)) == N.CS_OK
    small = np.zeros(3, np.int32)
    assert L.cs_build_bvh(c.np, N.dp(X), c.nt, N.ip(tri), N.ip(small), 3, ctypes.byref(nn)) == N.CS_ERR_CAPACITY
    return out.reshape(-1, 3)


def pattern(L, c):
    quad = np.ascontiguousarray(c.quad)
    nb = ctypes.c_int()
    rp = np.zeros(c.np + 1, np.int32)
    assert L.cs_build_pattern(c.np, c.nq, N.ip(quad), N.ip(rp), None, 0, ctypes.byref(nb)) == N.CS_OK
    ci = np.zeros(nb.value, np.int32)
    assert L.cs_build_pattern(c.np, c.nq, N.ip(quad), N.ip(rp), N.ip(ci), ci.size, ctypes.byref(nb)) == N.CS_OK
    return rp, ci


def test_fixtures(lib):
    for name, c in [("small_21", scene.config_small()),
                    ("fold_31", scene.square_cloth(31, 1.0, 0.4, sphere_radius=0.2, clearance=0.01, seed=11,
                                                   solver_kind=scene.SOLVER_CG, tol=1.0e-6, maxit=1000))]:
        arr = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
        assert np.array_equal(bvh(lib, c), arr["bvh_nodes"])
        rp, ci = pattern(lib, c)
        assert np.array_equal(rp, arr["row_ptr"]) and np.array_equal(ci, arr["col_idx"])


def test_batch_and_large_against_oracle(lib, oracle_port):
    cloths = scene.config_batch(count=12) + [scene.config_single_101()]
    for c in cloths:
        o = O.OracleCloth(oracle_port, c)
        assert np.array_equal(bvh(lib, c), o.bvh_nodes())
        rp, ci = pattern(lib, c)
        orp, oci = o.pattern()
        assert np.array_equal(rp, orp) and np.array_equal(ci, oci)


def test_bad_arguments(lib):
    tri = np.array([0, 1, 5], np.int32)
    X = np.zeros(9)
    nn = ctypes.c_int()
    assert lib.cs_build_bvh(3, N.dp(X), 1, N.ip(tri), None, 0, ctypes.byref(nn)) == N.CS_ERR_ARG
    assert lib.cs_build_bvh(0, N.dp(X), 1, N.ip(tri), None, 0, ctypes.byref(nn)) == N.CS_ERR_ARG
