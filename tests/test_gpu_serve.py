"""Serving (cs_server_*): continuous batching of scenes in one device arena.

A scene's final state is the same whether it ran alone (one cloth in its own
context) or in a mix whose membership changed while it ran: scenes joining,
scenes finishing, arenas packed on the side and swapped in.  Every reduction,
sort and level schedule of the frame is per cloth, so the tolerance here is
zero (bit-identical), for both precisions."""
import time

import numpy as np
import pytest

from cloth_sim_self_collision_gb300 import _native as N
from cloth_sim_self_collision_gb300 import scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cloth_sim_self_collision_gb300 import build
    build.build()


def _alone(cloth, nsteps, precision):
    from cloth_sim_self_collision_gb300.context import ClothContext
    ctx = ClothContext(0, precision)
    cid = ctx.add_cloth(cloth)
    ctx.step(nsteps)
    x, v = ctx.get_state(cid)
    ctx.close()
    return x, v


def _scenes():
    cg = dict(solver_kind=scene.SOLVER_CG, tol=1e-6, maxit=1000)
    return {
        "a": (scene.square_cloth(21, 1.0, 0.45, sphere_radius=0.3, seed=1, **cg), 40),
        "b": (scene.square_cloth(31, 1.0, 0.35, sphere_radius=0.2, rotation=0.7, seed=2, **cg), 70),
        "c": (scene.square_cloth(15, 1.0, 0.4, sphere_radius=0.25, rotation=1.3, seed=3, **cg), 25),
        "d": (scene.config_small(), 10),
    }


def _wait_frames(srv, n, limit=60.0):
    t = time.time()
    while srv.stats()["frames"] < n:
        assert time.time() - t < limit, "server made no progress"
        time.sleep(0.005)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_same_alone_and_in_mix(precision):
    from cloth_sim_self_collision_gb300.serve import Server
    sc = _scenes()
    ref = {k: _alone(c, n, precision) for k, (c, n) in sc.items()}
    with Server(0, precision, hbm_budget_bytes=16e9) as srv:
        req = {"b": srv.submit(*sc["b"])}
        _wait_frames(srv, 5)                      # b is running
        req["a"] = srv.submit(*sc["a"])
        _wait_frames(srv, 15)                     # a has joined b
        req["c"] = srv.submit(*sc["c"])
        req["d"] = srv.submit(*sc["d"])
        out = {k: srv.wait(r, timeout=600) for k, r in req.items()}
        st = srv.stats()
    for k, (x, v, info) in out.items():
        assert info["status"] == N.CS_OK and info["steps_done"] == sc[k][1], (k, info)
        assert np.array_equal(x, ref[k][0]), (precision, k, np.abs(x - ref[k][0]).max())
        assert np.array_equal(v, ref[k][1]), (precision, k, np.abs(v - ref[k][1]).max())
    # a joined while b ran, and c, d joined while a ran (arenas were swapped under it)
    ia, ib, ic = out["a"][2], out["b"][2], out["c"][2]
    assert ib["t_first_frame"] < ia["t_admit"] < ib["t_done"]
    assert ia["t_first_frame"] < ic["t_admit"] < ia["t_done"]
    assert st["rebuilds"] >= 3
    assert st["vertex_steps"] == sum(c.np * n for c, n in sc.values())
    assert st["finished"] == st["submitted"] == 4
    assert 0 < st["step_ms_p50"] <= st["step_ms_p99"] <= st["step_ms_max"]


def test_admission_by_budget():
    """Two scenes that do not fit the budget together run one after the other;
    a scene larger than the whole budget is refused at submission."""
    from cloth_sim_self_collision_gb300.serve import Server, scene_device_bytes
    c1 = scene.square_cloth(41, 1.0, 0.5, sphere_radius=0.3, seed=7, solver_kind=scene.SOLVER_CG, tol=1e-6,
                            maxit=1000)
    c2 = scene.square_cloth(41, 1.0, 0.6, sphere_radius=0.2, seed=8, solver_kind=scene.SOLVER_CG, tol=1e-6,
                            maxit=1000)
    nb = scene_device_bytes(c1)
    with Server(0, "mixed", hbm_budget_bytes=1.5 * nb) as srv:
        r1 = srv.submit(c1, 12)
        r2 = srv.submit(c2, 12)
        _, _, i1 = srv.wait(r1, timeout=600)
        x2, _, i2 = srv.wait(r2, timeout=600)
        assert i2["t_first_frame"] >= i1["t_done"]
        assert srv.stats()["peak_bytes"] <= 1.5 * nb
    ref = _alone(c2, 12, "mixed")
    assert np.array_equal(x2, ref[0])
    with Server(0, "mixed", hbm_budget_bytes=0.5 * nb) as srv:
        with pytest.raises(N.CsError) as e:
            srv.submit(c1, 5)
        assert e.value.code == N.CS_ERR_CAPACITY


def test_device_bytes_estimate():
    """The admission estimate is within 35% of what an arena really allocates."""
    import torch
    from cloth_sim_self_collision_gb300.context import ClothContext
    from cloth_sim_self_collision_gb300.serve import scene_device_bytes
    tiny = scene.square_cloth(5, 1.0, 0.5, solver_kind=scene.SOLVER_CG, maxit=1000)
    big = scene.square_cloth(121, 1.0, 0.5, solver_kind=scene.SOLVER_CG, maxit=1000)
    ctx = ClothContext(0, "mixed")
    t = ctx.add_cloth(tiny)
    ctx.step(1)
    torch.cuda.synchronize()
    f1 = torch.cuda.mem_get_info()[0]
    ctx.remove_cloth(t)
    ctx.add_cloth(big)
    ctx.step(1)
    torch.cuda.synchronize()
    f2 = torch.cuda.mem_get_info()[0]
    ctx.close()
    used = f1 - f2
    est = scene_device_bytes(big) - scene_device_bytes(tiny)
    assert 0.65 * used < est < 1.35 * used, (used, est)


def _wild(cloth, seed=0):
    """Initial velocities of 1e4 m/s in random directions: the cloth's swept boxes
    overlap everywhere at its first CCD pass, the host-made stand-in for a scene
    whose frames blew up."""
    return np.random.default_rng(seed).uniform(-1e4, 1e4, 3 * cloth.np)


def test_blown_up_cloth_is_isolated_in_a_context():
    from cloth_sim_self_collision_gb300.context import ClothContext
    cg = dict(solver_kind=scene.SOLVER_CG, tol=1e-6, maxit=1000)
    good = scene.square_cloth(21, 1.0, 0.45, sphere_radius=0.3, seed=1, **cg)
    bad = scene.square_cloth(31, 1.0, 0.6, sphere_radius=0.2, seed=2, **cg)
    ref = _alone(good, 12, "mixed")
    ctx = ClothContext(0, "mixed")
    ig = ctx.add_cloth(good)
    ib = ctx.add_cloth(bad)
    ctx.set_state(ib, v=_wild(bad))
    ctx.step(12)
    x, v = ctx.get_state(ig)
    sg, sb = ctx.stats(ig), ctx.stats(ib)
    ctx.close()
    assert sb["diverged"] == 1 and sg["diverged"] == 0
    assert np.array_equal(x, ref[0]) and np.array_equal(v, ref[1])


def test_blown_up_scene_fails_alone():
    """In a server, the blown-up scene ends with CS_ERR_DIVERGED and the scene
    sharing its arena finishes exactly as it does alone."""
    from cloth_sim_self_collision_gb300.serve import Server
    cg = dict(solver_kind=scene.SOLVER_CG, tol=1e-6, maxit=1000)
    good = scene.square_cloth(21, 1.0, 0.45, sphere_radius=0.3, seed=1, **cg)
    bad = scene.square_cloth(31, 1.0, 0.6, sphere_radius=0.2, seed=2, **cg)
    ref = _alone(good, 20, "mixed")
    with Server(0, "mixed", hbm_budget_bytes=16e9) as srv:
        rg = srv.submit(good, 20)
        rb = srv.submit(bad, 20, v=_wild(bad))
        x, v, info = srv.wait(rg, timeout=600)
        with pytest.raises(N.CsError) as e:
            srv.wait(rb, timeout=600)
        assert e.value.code == N.CS_ERR_DIVERGED
        st = srv.stats()
    assert st["diverged"] == 1 and st["finished"] == 2
    assert np.array_equal(x, ref[0]) and np.array_equal(v, ref[1])
