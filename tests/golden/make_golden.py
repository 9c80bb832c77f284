"""Generates the golden fixtures under tests/golden/ from the reference itself.

The reference has no tests or golden vectors of its own, so its sources are
compiled in place (oracle/Makefile target `ref`, the headless driver
oracle/ref_driver.cpp) and run here on seeded synthetic scenes.  The fixtures
record, per scene:

* the topology the reference derives (BVH nodes, matrix pattern, 1-ring);
* a SHA-256 of positions and velocities after every frame of the trajectory,
  and the per-frame counters (solver iterations, contact counts per pass);
* at one contact-rich frame, every stage of the step (assembly, ILU factor,
  PCG / CG, refits, contact sets, impulses, impact zones, velocity update):
  small integer results in full, floating-point arrays as SHA-256 digests;
* element-level known answers (CST, bending, obstacle contact) on random
  inputs, in full.

Run:  python tests/golden/make_golden.py   (needs the reference sources)
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cloth_sim_self_collision_gb300 import scene  # noqa: E402
from oracle import oracle as O  # noqa: E402


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def element_cases(lib, seed: int = 7, count: int = 24):
    rng = np.random.default_rng(seed)
    cst_in, cst_out, bend_in, bend_out, con_in, con_out = [], [], [], [], [], []
    for _ in range(count):
        C = rng.uniform(-1, 1, 9)
        c = C + rng.normal(0, 0.2, 9)
        lam, myu = rng.uniform(0.1, 3), rng.uniform(0.1, 3)
        W, dW, ddW = O.wdwddw_cst(lib, C, c, lam, myu)
        cst_in.append(np.concatenate([C, c, [lam, myu]]))
        cst_out.append(np.concatenate([[W], dW, ddW]))
        C4 = rng.uniform(-1, 1, 12)
        c4 = C4 + rng.normal(0, 0.2, 12)
        k = rng.uniform(1e-4, 1e-1)
        W, dW, ddW = O.wdwddw_bend(lib, C4, c4, k)
        bend_in.append(np.concatenate([C4, c4, [k]]))
        bend_out.append(np.concatenate([[W], dW, ddW]))
    prm = scene.Params(obs_radius=0.3, contact_clearance=0.01, stiff_contact=300.0)
    for kind in (scene.OBSTACLE_PLANE_Z, scene.OBSTACLE_SPHERE_SOLID, scene.OBSTACLE_SPHERE_HOLLOW):
        prm.obstacle_kind = kind
        prm.obs_center = (0.0, 0.0, 0.0) if kind != scene.OBSTACLE_PLANE_Z else (0.0, 0.0, -0.2)
        for _ in range(count // 3):
            p = rng.uniform(-0.35, 0.35, 3)
            W, dW, ddW = O.wdwddw_contact(lib, p, prm)
            con_in.append(np.concatenate([p, [kind]]))
            con_out.append(np.concatenate([[W], dW, ddW]))
    return dict(cst_in=np.array(cst_in), cst_out=np.array(cst_out), bend_in=np.array(bend_in),
                bend_out=np.array(bend_out), contact_in=np.array(con_in), contact_out=np.array(con_out))


def stage_record(sim, x, v, prm):
    """Every stage of one frame from state (x, v); floats as digests."""
    rec = {}
    vd, vc, b = sim.assemble(x, v)
    rec["assemble"] = [digest(vd), digest(vc), digest(b)]
    fd, fc, ns = sim.ilu()
    rec["ilu"] = [digest(fd), digest(fc), int(ns)]
    xs, conv, it = sim.pcg(b, 1e-6, 100)
    rec["pcg"] = [digest(xs), conv, it]
    xs, conv, it = sim.cg(b, 1e-6, 1000)
    rec["cg"] = [digest(xs), conv, it]
    x1, v1, st = sim.implicit(x, v)
    rec["implicit"] = [digest(x1), digest(v1), st["solver_iterations"], st["solver_conv"]]
    rec["refit_prx"] = digest(sim.refit_prx(x, prm.contact_clearance))
    rec["refit_ccd"] = digest(sim.refit_ccd(x, v1, prm.dt))
    prx = sim.contacts_prx(x, prm.contact_clearance)
    ccd = sim.contacts_ccd(x, v1, prm.dt, prm.contact_clearance)
    vi = sim.impulse_prx(x, v1, prx)
    rec["impulse_prx"] = digest(vi)
    ccd2 = sim.contacts_ccd(x, vi, prm.dt, prm.contact_clearance)
    rec["impulse_ccd"] = digest(sim.impulse_ccd(x, vi, ccd2))
    sim.riz_reset()
    sim.riz_add(ccd2)
    zones, nz = sim.riz_zones()
    rec["riz_apply"] = digest(sim.riz_apply(x, vi, vi))
    vr, st = sim.resolve(x, v1)
    rec["resolve"] = [digest(vr), {k: st[k] for k in ("n_prx", "n_ccd_passes", "n_ccd", "n_riz_passes",
                                                    "n_riz_last", "n_riz_total", "riz_nodes",
                                                    "impulse_applied")}]
    rec["update_velocity"] = digest(sim.update_velocity(x1, vr))
    arrays = dict(contacts_prx=prx, contacts_ccd=ccd, contacts_ccd_after_prx=ccd2, riz_zones=zones)
    rec["riz_count"] = int(nz)
    return rec, arrays


def make_scene_fixture(name: str, cloth, nsteps: int, probe_step: int):
    lib = O.OracleLib("ref")
    sim = O.OracleCloth(lib, cloth)
    rp, ci = sim.pattern()
    ei, ea = sim.edges()
    arrays = dict(bvh_nodes=sim.bvh_nodes(), row_ptr=rp, col_idx=ci, edge_index=ei, edge_array=ea)
    meta = dict(name=name, side=cloth.side, np=cloth.np, nt=cloth.nt, nq=cloth.nq,
                params=dict(cloth.params.__dict__), scene_digest=[digest(cloth.X0), digest(cloth.tri),
                                                                  digest(cloth.quad)],
                nsteps=nsteps, probe_step=probe_step, steps=[])
    for s in range(nsteps):
        if s == probe_step:
            arrays["probe_x"] = sim.x.copy()
            arrays["probe_v"] = sim.v.copy()
            rec, arr = stage_record(sim, sim.x.copy(), sim.v.copy(), cloth.params)
            meta["probe"] = rec
            arrays.update(arr)
        st = sim.step(1)[0]
        meta["steps"].append(dict(x=digest(sim.x), v=digest(sim.v), stats={
            k: st[k] for k in ("solver_iterations", "n_prx", "n_ccd_passes", "n_ccd", "n_riz_passes",
                               "n_riz_last", "n_riz_total", "riz_nodes", "impulse_applied", "ilu_singular")}))
    arrays["final_x"] = sim.x.copy()
    arrays["final_v"] = sim.v.copy()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(meta, f, indent=1)
    sim.close()


def main():
    O.build("ref")
    lib = O.OracleLib("ref")
    np.savez_compressed(os.path.join(HERE, "elements.npz"), **element_cases(lib))
    # 21x21 sheet over a sphere (ILU(0)-PCG); frame 45 carries proximity, CCD and RIZ work
    make_scene_fixture("small_21", scene.config_small(), nsteps=300, probe_step=45)
    # a 31x31 sheet dropped lower so it folds early (CG solver)
    c = scene.square_cloth(31, 1.0, 0.4, sphere_radius=0.2, clearance=0.01, seed=11,
                           solver_kind=scene.SOLVER_CG, tol=1.0e-6, maxit=1000)
    make_scene_fixture("fold_31", c, nsteps=120, probe_step=60)


if __name__ == "__main__":
    main()
