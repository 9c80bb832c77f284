"""The oracle restatement against the golden fixtures recorded from the
reference (tests/golden/make_golden.py).  CPU only."""
import json
import os

import numpy as np
import pytest

from cloth_sim_self_collision_gb300 import scene
from oracle import oracle as O
from tests.golden.make_golden import digest, stage_record

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        meta = json.load(f)
    arr = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    return meta, arr


def scene_for(name):
    if name == "small_21":
        return scene.config_small()
    return scene.square_cloth(31, 1.0, 0.4, sphere_radius=0.2, clearance=0.01, seed=11,
                              solver_kind=scene.SOLVER_CG, tol=1.0e-6, maxit=1000)


def test_element_known_answers(oracle_port):
    g = dict(np.load(os.path.join(GOLDEN, "elements.npz")))
    for inp, out in zip(g["cst_in"], g["cst_out"]):
        W, dW, ddW = O.wdwddw_cst(oracle_port, inp[:9], inp[9:18], inp[18], inp[19])
        assert np.array_equal(np.concatenate([[W], dW, ddW]), out)
    for inp, out in zip(g["bend_in"], g["bend_out"]):
        W, dW, ddW = O.wdwddw_bend(oracle_port, inp[:12], inp[12:24], inp[24])
        assert np.array_equal(np.concatenate([[W], dW, ddW]), out)
    prm = scene.Params(obs_radius=0.3, contact_clearance=0.01, stiff_contact=300.0)
    for inp, out in zip(g["contact_in"], g["contact_out"]):
        prm.obstacle_kind = int(inp[3])
        prm.obs_center = (0.0, 0.0, 0.0) if prm.obstacle_kind != scene.OBSTACLE_PLANE_Z else (0.0, 0.0, -0.2)
        W, dW, ddW = O.wdwddw_contact(oracle_port, inp[:3], prm)
        assert np.array_equal(np.concatenate([[W], dW, ddW]), out)


@pytest.mark.parametrize("name", ["small_21", "fold_31"])
def test_scene_generator_pinned(name):
    meta, _ = load(name)
    c = scene_for(name)
    assert [digest(c.X0), digest(c.tri), digest(c.quad)] == meta["scene_digest"]


@pytest.mark.parametrize("name", ["small_21", "fold_31"])
def test_topology(oracle_port, name):
    meta, arr = load(name)
    sim = O.OracleCloth(oracle_port, scene_for(name))
    assert np.array_equal(sim.bvh_nodes(), arr["bvh_nodes"])
    rp, ci = sim.pattern()
    assert np.array_equal(rp, arr["row_ptr"]) and np.array_equal(ci, arr["col_idx"])
    ei, ea = sim.edges()
    assert np.array_equal(ei, arr["edge_index"]) and np.array_equal(ea, arr["edge_array"])


@pytest.mark.parametrize("name", ["small_21", "fold_31"])
def test_stages_at_probe_frame(oracle_port, name):
    meta, arr = load(name)
    c = scene_for(name)
    sim = O.OracleCloth(oracle_port, c)
    rec, a = stage_record(sim, arr["probe_x"], arr["probe_v"], c.params)
    expect = meta["probe"]
    for k in expect:
        assert rec[k] == expect[k], k
    for k, v in a.items():
        assert np.array_equal(v, arr[k]), k


@pytest.mark.parametrize("name", ["small_21", "fold_31"])
def test_trajectory_bit_exact(oracle_port, name):
    meta, arr = load(name)
    sim = O.OracleCloth(oracle_port, scene_for(name))
    for s, rec in enumerate(meta["steps"]):
        st = sim.step(1)[0]
        assert digest(sim.x) == rec["x"] and digest(sim.v) == rec["v"], f"frame {s}"
        for k, v in rec["stats"].items():
            assert st[k] == v, (s, k)
    assert np.array_equal(sim.x, arr["final_x"]) and np.array_equal(sim.v, arr["final_v"])
