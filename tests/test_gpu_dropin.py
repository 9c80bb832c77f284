"""The C++ drop-in (cloth_sim_self_collision_gb300/dropin): a driver written
against the reference's own API (StepTime_InternalDynamicsILU,
GetIntermidiateVelocityContactResolved, UpdateIntermidiateVelocity,
MakeBVHTopology_TopDown, the container classes) is compiled against the
drop-in headers and run on the GPU; with the drop-in's defaults (the
reference's hard-coded solver settings, serial inner products) its frames equal
the oracle's bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from cloth_sim_self_collision_gb300 import build, scene
from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(build.LIB_DIR)


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    build.build()
    exe = str(tmp_path_factory.mktemp("dropin") / "driver")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-o", exe,
                    os.path.join(HERE, "dropin", "driver.cpp"), "-I", os.path.join(PKG, "dropin"),
                    "-L", build.LIB_DIR, "-lclothgpu_dropin", "-lclothgpu", "-Wl,-rpath," + build.LIB_DIR],
                   check=True)
    return exe


def write_scene(path, c, use_cg):
    p = c.params
    prm = np.array([p.dt, p.lam, p.myu, p.stiff_bend, *p.gravity, p.mass_point, p.stiff_contact,
                    p.contact_clearance, *p.obs_center, p.obs_radius, 1.0 if use_cg else 0.0])
    with open(path, "wb") as f:
        for a, dt in ((c.X0, np.float64), (c.tri, np.int32), (c.quad, np.int32), (prm, np.float64)):
            a = np.ascontiguousarray(a, dt)
            f.write(np.int64(a.size).tobytes())
            f.write(a.tobytes())


@pytest.mark.parametrize("name,frames", [("small_21", 60), ("fold_31", 45)])
def test_dropin_frames_bit_exact(driver, oracle_port, tmp_path, name, frames):
    if name == "small_21":
        c = scene.config_small()
        use_cg = False
        c.params.solver_kind, c.params.tol, c.params.maxit = scene.SOLVER_ILU_PCG, 1e-4, 100
    else:
        c = scene.square_cloth(31, 1.0, 0.4, sphere_radius=0.2, clearance=0.01, seed=11)
        use_cg = True
        c.params.solver_kind, c.params.tol, c.params.maxit = scene.SOLVER_CG, 1e-4, 1000
    sc, out = str(tmp_path / "scene.bin"), str(tmp_path / "out.bin")
    write_scene(sc, c, use_cg)
    subprocess.run([driver, sc, str(frames), out], check=True, timeout=600)
    res = np.fromfile(out, dtype=np.float64)
    x, v = res[: c.np * 3], res[c.np * 3:]
    orc = O.OracleCloth(oracle_port, c)
    orc.step(frames)
    assert np.array_equal(x, orc.x) and np.array_equal(v, orc.v), np.abs(x - orc.x).max()
