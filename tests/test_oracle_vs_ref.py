"""The oracle restatement against the reference built from its own sources,
live, on inputs beyond the fixtures.  Skipped where the reference is absent."""
import numpy as np
import pytest

from cloth_sim_self_collision_gb300 import scene
from oracle import oracle as O


def test_elements_random(oracle_port, oracle_ref):
    rng = np.random.default_rng(1234)
    for _ in range(200):
        C = rng.uniform(-1, 1, 9)
        c = C + rng.normal(0, 0.5, 9)
        a = O.wdwddw_cst(oracle_port, C, c, 0.7, 1.3)
        b = O.wdwddw_cst(oracle_ref, C, c, 0.7, 1.3)
        assert a[0] == b[0] and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
        C4 = rng.uniform(-1, 1, 12)
        c4 = C4 + rng.normal(0, 0.5, 12)
        a = O.wdwddw_bend(oracle_port, C4, c4, 0.01)
        b = O.wdwddw_bend(oracle_ref, C4, c4, 0.01)
        assert a[0] == b[0] and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


@pytest.mark.parametrize("side,steps", [(61, 3), (101, 2)])
def test_large_sheet_steps(oracle_port, oracle_ref, side, steps):
    c = scene.square_cloth(side, 2.0, 1.0, sphere_radius=0.25, solver_kind=scene.SOLVER_CG,
                           tol=1e-6, maxit=1000)
    a = O.OracleCloth(oracle_port, c)
    b = O.OracleCloth(oracle_ref, c)
    assert np.array_equal(a.bvh_nodes(), b.bvh_nodes())
    for _ in range(steps):
        assert a.step(1) == b.step(1)
        assert np.array_equal(a.x, b.x) and np.array_equal(a.v, b.v)


def test_batch_instances_topology(oracle_port, oracle_ref):
    for c in scene.config_batch(count=6):
        a = O.OracleCloth(oracle_port, c)
        b = O.OracleCloth(oracle_ref, c)
        assert np.array_equal(a.bvh_nodes(), b.bvh_nodes())
        assert a.step(1) == b.step(1)
        assert np.array_equal(a.x, b.x)


def test_vertex_normals_match_reference(oracle_port, oracle_ref):
    """MakeNormal: the restatement equals the reference's UnitNormalAreaTri3D loop
    bit for bit, on a flat sheet and on a folded state."""
    from cloth_sim_self_collision_gb300 import scene
    c = scene.square_cloth(31, 1.0, 0.4, sphere_radius=0.2, clearance=0.01, seed=11,
                           solver_kind=scene.SOLVER_CG, tol=1.0e-6, maxit=1000)
    a = O.OracleCloth(oracle_port, c)
    b = O.OracleCloth(oracle_ref, c)
    a.step(40)
    for x in (c.X0, a.x):
        na, nb = a.vertex_normals(x), b.vertex_normals(x)
        assert np.array_equal(na, nb)
        assert np.allclose(np.linalg.norm(na.reshape(-1, 3), axis=1), 1.0)


DEMO = dict(lam=0.0, myu=30.0, stiff_bend=1e-2, dt=0.01, gravity=(0.0, 0.05, -10.0))


@pytest.mark.parametrize("obstacle,center,radius,material", [
    (scene.OBSTACLE_PLANE_Z, (0.0, 0.0, -0.1), 0.0, "demo"),
    (scene.OBSTACLE_SPHERE_HOLLOW, (0.5, 0.0, 2.0), 1.7, "demo"),
    (scene.OBSTACLE_SPHERE_SOLID, (0.0, 0.0, 0.0), 0.3, "demo"),
    (scene.OBSTACLE_PLANE_Z, (0.0, 0.0, 0.3), 0.0, "config"),
    (scene.OBSTACLE_NONE, (0.0, 0.0, 0.0), 0.0, "config"),
])
def test_obstacles_and_materials(oracle_port, oracle_ref, obstacle, center, radius, material):
    """Every obstacle descriptor (the demo's plane and inside-out sphere, the
    benchmark's solid sphere, none) with the demo's and the configurations'
    material: the restatement's frames equal the reference's bit for bit,
    through first contact with the obstacle."""
    # the demo's material makes ILU(0) stall on this sheet: the reference's CG, as
    # the serving scenes use it; the configurations' material factorises
    if material == "demo":
        kw = dict(DEMO, solver_kind=scene.SOLVER_CG, tol=1e-6, maxit=1000)
    else:
        kw = dict(solver_kind=scene.SOLVER_ILU_PCG, tol=1e-4, maxit=100)
    c = scene.square_cloth(21, 1.0, 0.4, sphere_radius=radius, seed=5, density=0.04 if material == "demo" else 1.0,
                           obstacle_kind=obstacle, obs_center=center, **kw)
    a = O.OracleCloth(oracle_port, c)
    b = O.OracleCloth(oracle_ref, c)
    touched = False
    for _ in range(45):
        sa, sb = a.step(1), b.step(1)
        assert sa == sb
        assert np.array_equal(a.x, b.x) and np.array_equal(a.v, b.v)
    if obstacle == scene.OBSTACLE_PLANE_Z:
        touched = a.x.reshape(-1, 3)[:, 2].min() < center[2] + 0.02
    elif obstacle == scene.OBSTACLE_SPHERE_HOLLOW:
        touched = np.linalg.norm(a.x.reshape(-1, 3) - np.array(center), axis=1).max() > radius - 0.02
    elif obstacle == scene.OBSTACLE_SPHERE_SOLID:
        touched = np.linalg.norm(a.x.reshape(-1, 3), axis=1).min() < radius + 0.02
    else:
        touched = True
    assert touched


def test_matrix_functions_match_reference(oracle_port, oracle_ref):
    """MatVec with general alpha / beta, Solve_CG and Solve_PCG with the residual
    they leave in r_vec, DoILUDecomp and CPreconditionerILU::Solve: the
    restatement equals the reference bit for bit on an assembled system,
    including a CG cut off by its iteration cap."""
    c = scene.config_small()
    a = O.OracleCloth(oracle_port, c)
    b = O.OracleCloth(oracle_ref, c)
    a.step(30)
    x, v = a.x.copy(), a.v.copy()
    va, vb = a.assemble(x, v), b.assemble(x, v)
    for p, q in zip(va, vb):
        assert np.array_equal(p, q)
    rhs = va[2]
    rng = np.random.default_rng(7)
    xs, ys = rng.normal(size=rhs.size), rng.normal(size=rhs.size)
    for alpha, beta in ((1.0, 0.0), (0.5, 2.0), (-1.25, 0.75)):
        assert np.array_equal(a.matvec(alpha, xs, beta, ys), b.matvec(alpha, xs, beta, ys))
    for tol, maxit in ((1e-6, 1000), (1e-6, 5)):
        ra, rb = a.cg(rhs, tol, maxit), b.cg(rhs, tol, maxit)
        assert np.array_equal(ra[0], rb[0]) and ra[1:] == rb[1:]
        assert np.array_equal(a.last_residual(), b.last_residual())
    fa, fb = a.ilu(), b.ilu()
    assert np.array_equal(fa[0], fb[0]) and np.array_equal(fa[1], fb[1]) and fa[2] == fb[2]
    assert np.array_equal(a.ilu_solve(rhs), b.ilu_solve(rhs))
    pa, pb = a.pcg(rhs, 1e-6, 100), b.pcg(rhs, 1e-6, 100)
    assert np.array_equal(pa[0], pb[0]) and pa[1:] == pb[1:]
    assert np.array_equal(a.last_residual(), b.last_residual())


def test_geometry_functions_match_reference(oracle_port, oracle_ref):
    """DistanceFaceVertex, DistanceEdgeEdge (both branches) and
    FindCoplanerInterp (roots, no roots, the quadratic case) bit for bit."""
    rng = np.random.default_rng(99)
    for k in range(300):
        p = rng.uniform(-1, 1, 12)
        if k % 5 == 0:  # parallel edges
            p[9:12] = p[6:9] + 0.5 * (p[3:6] - p[0:3])
        assert O.distance_fv(oracle_port, p) == O.distance_fv(oracle_ref, p)
        assert O.distance_ee(oracle_port, p) == O.distance_ee(oracle_ref, p)
        e = p + rng.normal(0, 0.3 if k % 3 else 1e-3, 12)
        if k % 7 == 0:  # equal displacement of all points: the cubic degenerates
            e = p + np.tile(rng.normal(0, 0.2, 3), 4)
        assert O.coplanar_time(oracle_port, p, e) == O.coplanar_time(oracle_ref, p, e)


def test_ccd_tests_match_reference(oracle_port, oracle_ref):
    """IsContact_FV_CCD and IsContact_EE_CCD on the configurations the
    certificate tests use (sheet patches, crossing sheets, exactly flat
    sheets, random): the restatement's decisions equal the reference's."""
    import test_ccd_certificates as T
    for kind in ("fv", "ee"):
        for i, (name, make) in enumerate(T.SCENARIOS.items()):
            cfg = make(np.random.default_rng(500 + 10 * i + (kind == "ee")), kind)
            if kind == "fv":
                box = np.array([-0.3, -0.3, -0.3, 0.3, 0.3, 0.3])
                a, b = O.fv_ccd(oracle_port, cfg, box), O.fv_ccd(oracle_ref, cfg, box)
            else:
                a, b = O.ee_ccd(oracle_port, cfg), O.ee_ccd(oracle_ref, cfg)
            assert np.array_equal(a, b), (kind, name, np.nonzero(a != b)[0][:5])
            assert 0 < b.sum() or name in ("sheet", "flat")
