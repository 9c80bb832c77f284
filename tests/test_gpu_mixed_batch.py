"""The benchmarked path against the FP64 oracle, frame by frame, in contact.

The batched workload runs CS_PREC_MIXED: FP32 CG inside FP64 iterative
refinement, with collision in FP64.  Its stated bound, per frame from the same
start state as the oracle:

* positions:  max |x - x_oracle| <= MIXED_RTOL * max(1, max |x_oracle|)
* velocities, as the position change they make over the frame:
              max |v - v_oracle| * dt <= MIXED_RTOL * max(1, max |x_oracle|)
* every detection of the frame (proximity, each CCD pass, each impact-zone
  pass) finds the same ordered contact list as the oracle's (compared through
  the contact log: kind, count and a 64-bit digest of the list).

The plain FP64 path meets the same checks at FP64_RTOL with tree-summed inner
products, and bit for bit with serial ones (CS_FLAG_EXACT_DOTS).

Start states: the first 24 sheets of the batched workload (sides 19-69, four of
them 61 or more vertices a side) stepped on the GPU in FP64 with serial inner
products, which reproduces the reference bit for bit; frames 10 and 20 are in
free fall or first touch, 30 and 40 in heavy contact (several CCD passes and
impact zones).  From each state the oracle steps one frame in a pool of host
processes (a full oracle trajectory of the 69 x 69 sheet through contact takes
minutes)."""
import dataclasses

import numpy as np
import pytest

from cloth_sim_self_collision_gb300 import scene
from oracle import pool

pytestmark = pytest.mark.gpu

MIXED_RTOL = 1e-6
FP64_RTOL = 1e-9
FRAMES = (10, 20, 30, 40)
N_CLOTHS = 24


def rel_err(a, b):
    return float(np.max(np.abs(a - b), initial=0.0) / max(1.0, np.max(np.abs(b), initial=0.0)))


def with_flags(c, flags):
    return dataclasses.replace(c, params=dataclasses.replace(c.params, flags=flags))


@pytest.fixture(scope="module")
def batch():
    """(cloths, {frame: [(x, v) per cloth]}, {frame: [oracle result per cloth]})"""
    from cloth_sim_self_collision_gb300 import build
    build.build()
    from cloth_sim_self_collision_gb300.context import ClothContext
    cl = scene.config_batch(count=N_CLOTHS)
    exact = [with_flags(c, 1) for c in cl]
    ctx = ClothContext(0, "fp64")
    states = {}
    try:
        ids = [ctx.add_cloth(c) for c in exact]
        f = 0
        for k in FRAMES:
            ctx.step(k - f)
            f = k
            states[k] = [ctx.get_state(i) for i in ids]
    finally:
        ctx.close()
    jobs, cost = [], []
    for k in FRAMES:
        for i, c in enumerate(cl):
            x, v = states[k][i]
            jobs.append((c, x, v, 1, True, 0))
            cost.append(c.np * (4 if k >= 30 else 1))
    res = pool.run_jobs(jobs, cost=cost)
    nxt, j = {}, 0
    for k in FRAMES:
        nxt[k] = []
        for _ in cl:
            nxt[k].append(res[j][-1])
            j += 1
    return cl, states, nxt


def step_from(prec, cloths, states, flags=0):
    """One frame of every cloth from each start state: {frame: [(x, v, log, stats)]}"""
    from cloth_sim_self_collision_gb300.context import ClothContext
    ctx = ClothContext(0, prec)
    out = {}
    try:
        ids = [ctx.add_cloth(with_flags(c, flags)) for c in cloths]
        ctx.log_contacts(True)
        for k, st in states.items():
            for i, (x, v) in zip(ids, st):
                ctx.set_state(i, x, v)
            ctx.step(1)
            out[k] = [ctx.get_state(i) + (ctx.contact_log(i), ctx.stats(i)) for i in ids]
    finally:
        ctx.close()
    return out


def check(prec_out, cl, nxt, rtol, exact=False):
    """Compares every (frame, cloth) with the oracle; collects all violations
    before failing, so one run shows the whole picture.  Velocities are held to
    the position bound per frame: |dv| dt <= rtol max(1, max |x|)."""
    worst_x = worst_v = 0.0
    detections = contacts = 0
    bad = []
    for k, rows in prec_out.items():
        for i, (x, v, log, st) in enumerate(rows):
            _, xo, vo, logo, sto = nxt[k][i]
            dt = cl[i].params.dt
            if exact and not (np.array_equal(x, xo) and np.array_equal(v, vo)):
                bad.append((k, i, "not bit-exact"))
            if log != logo:
                first = next((j for j, (a, b) in enumerate(zip(log, logo)) if a != b), min(len(log), len(logo)))
                bad.append((k, i, cl[i].side, "contact log differs at detection", first,
                            [(a[0], a[1]) for a in log], [(a[0], a[1]) for a in logo]))
                continue
            scale = max(1.0, np.max(np.abs(xo)))
            ex = float(np.max(np.abs(x - xo)) / scale)
            ev = float(np.max(np.abs(v - vo)) * dt / scale)
            worst_x, worst_v = max(worst_x, ex), max(worst_v, ev)
            if ex > rtol or ev > rtol:
                bad.append((k, i, cl[i].side, "x", ex, "v*dt", ev))
            detections += len(log)
            contacts += sum(c for _, c, _ in log)
    print(f"worst x {worst_x:.2e}, worst |dv| dt {worst_v:.2e}, {detections} detections with "
          f"{contacts} contacts identical; violations: {bad}")
    assert not bad, bad
    return worst_x, worst_v, detections, contacts


def test_batch_states_reach_contact(batch):
    """The chosen frames exercise every stage: proximity contacts, several CCD
    passes and impact zones (counted on the oracle's frames)."""
    cl, _, nxt = batch
    stats = [r[4] for k in (30, 40) for r in nxt[k]]
    assert sum(s["n_prx"] for s in stats) > 1000
    assert sum(s["n_ccd_passes"] >= 2 for s in stats) >= 8
    assert sum(s["n_riz_passes"] > 0 for s in stats) >= 4
    assert sum(c.side >= 61 for c in cl) >= 4


def test_batch_fp64_exact_frames_bit_exact(batch):
    cl, states, nxt = batch
    out = step_from("fp64", cl, states, flags=1)
    check(out, cl, nxt, 0.0, exact=True)


def test_batch_fp64_frames(batch):
    cl, states, nxt = batch
    out = step_from("fp64", cl, states)
    wx, wv, nd, nc = check(out, cl, nxt, FP64_RTOL)
    print(f"fp64 batch frames: worst x {wx:.2e} v {wv:.2e}, {nd} detections, {nc} contacts identical")


def test_batch_mixed_frames(batch):
    """The benchmarked precision: within MIXED_RTOL of the FP64 oracle, with
    identical contact lists in every detection of every frame."""
    cl, states, nxt = batch
    out = step_from("mixed", cl, states)
    wx, wv, nd, nc = check(out, cl, nxt, MIXED_RTOL)
    print(f"mixed batch frames: worst x {wx:.2e} v {wv:.2e}, {nd} detections, {nc} contacts identical")


def test_batch_fp64_trajectory_through_contact():
    """Eight sheets of the batch (sides 19-45) in one FP64 arena with serial
    inner products, 60 frames from rest through first contact and draping: the
    state every 10 frames equals the oracle's own trajectory bit for bit."""
    from cloth_sim_self_collision_gb300 import build
    build.build()
    from cloth_sim_self_collision_gb300.context import ClothContext
    allc = scene.config_batch(count=N_CLOTHS)
    pick = [0, 1, 3, 4, 10, 14, 22, 23]
    cl = [with_flags(allc[i], 1) for i in pick]
    orc = pool.run_jobs([(c, None, None, 60, False, 10) for c in cl], cost=[c.np for c in cl])
    ctx = ClothContext(0, "fp64")
    try:
        ids = [ctx.add_cloth(c) for c in cl]
        touched = 0
        for f in range(10, 61, 10):
            ctx.step(10)
            for n, i in enumerate(ids):
                x, v = ctx.get_state(i)
                fo, xo, vo, _, _ = orc[n][f // 10 - 1]
                assert fo == f
                assert np.array_equal(x, xo) and np.array_equal(v, vo), (f, pick[n])
                touched += ctx.stats(i)["n_prx"] > 0
        assert touched >= 8
    finally:
        ctx.close()
