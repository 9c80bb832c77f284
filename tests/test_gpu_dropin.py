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


def _read_vecs(path, kinds):
    out = []
    with open(path, "rb") as f:
        for dt in kinds:
            n = int(np.frombuffer(f.read(8), np.int64)[0])
            out.append(np.frombuffer(f.read(n * np.dtype(dt).itemsize), dt).copy())
    return out


def _mearge_restated(c, rp, ci):
    """Mearge / SetBoundaryCondition of the driver's element matrices, restated
    (matrix_square_sparse.cpp:88-138, 272-302)."""
    n, nq = c.np, c.nq
    vd = np.zeros((n, 9))
    vc = np.zeros((len(ci), 9))
    quad = c.quad.reshape(-1, 4)
    for q in range(0, nq, 3):
        k = np.arange(16 * 9)
        emat = (0.001 * ((q * 131 + k * 17) % 97) - 0.05).reshape(4, 4, 9)
        for a in range(4):
            row = quad[q, a]
            slots = {ci[s]: s for s in range(rp[row], rp[row + 1])}
            for b in range(4):
                if a == b:
                    vd[row] += emat[a, b]
                elif quad[q, b] in slots:
                    vc[slots[quad[q, b]]] += emat[a, b]
    bc = np.zeros(n, bool)
    bc[::7] = True
    for i in np.nonzero(bc)[0]:
        vd[i] = np.eye(3).reshape(9)
        vc[rp[i]:rp[i + 1]] = 0.0
    vc[bc[ci]] = 0.0
    return vd.reshape(-1), vc.reshape(-1)


def test_dropin_lower_level_functions(driver, oracle_port, tmp_path):
    """The lower-level functions of the reference's headers through the drop-in,
    each against the oracle on the same inputs, bit for bit: BVH refits
    (BuildBoundingBoxChild_Prx / _CCD), contact searches (GetContactElement_*),
    MatVec, Solve_CG (converged and cut off by its cap, with the residual it
    leaves), DoILUDecomp, CPreconditionerILU::Solve, Solve_PCG, Mearge with
    SetBoundaryCondition, DistanceFaceVertex, DistanceEdgeEdge and
    FindCoplanerInterp."""
    c = scene.config_small()
    c.params.solver_kind, c.params.tol, c.params.maxit = scene.SOLVER_ILU_PCG, 1e-4, 100
    orc = O.OracleCloth(oracle_port, c)
    orc.step(40)  # draped over the sphere: contacts in both searches
    x, v = orc.x.copy(), orc.v.copy()
    vd, vc, b = orc.assemble(x, v)
    rng = np.random.default_rng(5)
    geo = rng.uniform(-1, 1, 12 * 64)
    geo[12 * 32: 12 * 40].reshape(8, 12)[:, 9:12] = (geo[12 * 32: 12 * 40].reshape(8, 12)[:, 6:9] + 0.3 *
                                                      (geo[12 * 32: 12 * 40].reshape(8, 12)[:, 3:6] -
                                                       geo[12 * 32: 12 * 40].reshape(8, 12)[:, 0:3]))
    geo_e = geo + rng.normal(0, 0.3, geo.size)
    sc, st, out = str(tmp_path / "scene.bin"), str(tmp_path / "state.bin"), str(tmp_path / "out.bin")
    write_scene(sc, c, False)
    with open(st, "wb") as f:
        for a in (x, v, vd, vc, b, geo, geo_e):
            a = np.ascontiguousarray(a, np.float64)
            f.write(np.int64(a.size).tobytes())
            f.write(a.tobytes())
    subprocess.run([driver, "lower", sc, st, out], check=True, timeout=600)
    d, i = np.float64, np.int32
    (bp, cp, bc_, cc, y1, y2, u1, r1, s1, u2, r2, s2, fd, fc, z, up, rpv, sp, md, mc, g) = _read_vecs(
        out, [d, i, d, i, d, d, d, d, d, d, d, d, d, d, d, d, d, d, d, d, d])
    dt, delta = c.params.dt, c.params.contact_clearance
    assert np.array_equal(bp.reshape(-1, 7), orc.refit_prx(x, delta))
    prx = orc.contacts_prx(x, delta)
    assert len(prx) > 0 and np.array_equal(cp.reshape(-1, 5), prx)
    assert np.array_equal(bc_.reshape(-1, 7), orc.refit_ccd(x, v, dt))
    assert np.array_equal(cc.reshape(-1, 5), orc.contacts_ccd(x, v, dt, delta))
    orc.assemble(x, v)
    assert np.array_equal(y1, orc.matvec(1.0, x, 0.0, v))
    assert np.array_equal(y2, orc.matvec(0.5, x, 2.0, v))
    for (u, r, s), maxit in (((u1, r1, s1), 1000), ((u2, r2, s2), 5)):
        xo, conv, it = orc.cg(b, 1e-6, maxit)
        assert np.array_equal(u, xo) and np.array_equal(r, orc.last_residual())
        assert s[0] == conv and int(s[1]) == it
    fdo, fco, _ = orc.ilu()
    assert np.array_equal(fd, fdo) and np.array_equal(fc, fco)
    assert np.array_equal(z, orc.ilu_solve(b))
    xo, conv, it = orc.pcg(b, 1e-6, 100)
    assert np.array_equal(up, xo) and np.array_equal(rpv, orc.last_residual())
    assert sp[0] == conv and int(sp[1]) == it
    rp, ci = orc.pattern()
    md_o, mc_o = _mearge_restated(c, rp, ci)
    assert np.array_equal(md, md_o) and np.array_equal(mc, mc_o)
    g = g.reshape(-1, 7)
    for k in range(64):
        p, e = geo[12 * k: 12 * k + 12], geo_e[12 * k: 12 * k + 12]
        assert tuple(g[k, 0:3]) == O.distance_fv(oracle_port, p)
        assert tuple(g[k, 3:6]) == O.distance_ee(oracle_port, p)
        assert g[k, 6] == O.coplanar_time(oracle_port, p, e)
