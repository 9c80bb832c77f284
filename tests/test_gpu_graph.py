"""Frames captured as a CUDA graph (cs_set_frame_mode CS_FRAME_GRAPH, the
default) against host-driven frames (CS_FRAME_HOST) on the same cloths: every
state and every frame counter equal bit for bit, in free fall and through
contact, for both precisions and for the ILU(0) sheet, and one host launch per
graph frame.  A graph frame whose contact lists outgrow the graph's fixed sort
sizes is restored and re-run host-driven, and a new graph is captured: forced
here with small minimum sizes, with the frames still equal bit for bit."""
import os

import numpy as np
import pytest

from cloth_sim_self_collision_gb300 import scene

pytestmark = pytest.mark.gpu

STAT_KEYS = ("solver_iterations", "n_prx", "n_ccd", "n_ccd_passes", "n_riz_passes", "n_riz_last", "n_riz_total",
             "riz_nodes", "impulse_applied", "ilu_singular", "diverged")


def run(cloths, prec, graph, frames, every=10):
    from cloth_sim_self_collision_gb300 import build
    build.build()
    from cloth_sim_self_collision_gb300.context import ClothContext
    ctx = ClothContext(0, prec)
    try:
        ctx.frame_mode(graph)
        ids = [ctx.add_cloth(c) for c in cloths]
        ctx.step(1)
        launches0 = ctx.launch_count()
        states, stats, per_frame = [], [], []
        for f in range(2, frames + 1):
            l0 = ctx.launch_count()
            ctx.step(1)
            per_frame.append(ctx.launch_count() - l0)
            stats.append([{k: ctx.stats(i)[k] for k in STAT_KEYS} for i in ids])
            if f % every == 0:
                states.append([ctx.get_state(i) for i in ids])
        return states, stats, ctx.frame_counts(), ctx.launch_count() - launches0, frames - 1, per_frame
    finally:
        ctx.close()


def same(a, b):
    for sa, sb in zip(a[0], b[0]):
        for (xa, va), (xb, vb) in zip(sa, sb):
            if not (np.array_equal(xa, xb) and np.array_equal(va, vb)):
                return False
    return a[1] == b[1]


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_graph_frames_equal_host_frames(prec):
    cl = scene.config_batch(count=16)
    g = run(cl, prec, True, 40)
    h = run(cl, prec, False, 40)
    assert same(g, h)
    assert g[2]["graph_frames"] >= g[4] - g[2]["overflows"] and h[2]["graph_frames"] == 0
    touched = sum(s["n_prx"] > 0 for fr in g[1] for s in fr)
    assert touched > 20, touched
    # one graph launch per graph frame; only the frames that outgrew the graph's
    # fixed sizes (re-run host-driven) issue kernel launches from the host
    print(f"{prec}: host launches per frame graph {g[3] / g[4]:.1f}, host-driven {h[3] / h[4]:.1f}; {g[2]}")
    # (frames before the first capture count as graph frames once captured)
    assert g[3] <= g[4] + g[2]["overflows"] * max(h[5])
    assert sum(n == 1 for n in g[5]) >= g[4] - g[2]["overflows"] - 1


def test_graph_frames_ilu_sheet():
    c = scene.config_small()
    g = run([c], "fp64", True, 120)
    h = run([c], "fp64", False, 120)
    assert same(g, h)
    assert g[2]["graph_frames"] > 0


def test_graph_overflow_rerun_and_recapture(monkeypatch):
    monkeypatch.setenv("CLOTHGPU_GRAPH_SORT_MIN", "64")
    monkeypatch.setenv("CLOTHGPU_GRAPH_ZONE_MIN", "16")
    cl = scene.config_batch(count=16)
    g = run(cl, "mixed", True, 40)
    h = run(cl, "mixed", False, 40)
    assert same(g, h)
    assert g[2]["overflows"] > 0 and g[2]["captures"] > 1 and g[2]["graph_frames"] > 0, g[2]


def test_narrow_register_variants_equal(monkeypatch):
    """The FP64 narrow-phase kernels capped at 128 registers (a variant the
    autotuner may pick) find the same contacts: frames equal bit for bit."""
    cl = scene.config_batch(count=16)
    a = run(cl, "mixed", True, 40)
    monkeypatch.setenv("CLOTHGPU_NARROW_REGS", "128")
    b = run(cl, "mixed", True, 40)
    assert same(a, b)
    assert sum(sum(s["n_ccd"]) > 0 for fr in b[1] for s in fr) > 0


@pytest.mark.parametrize("graph", [True, False])
def test_impulse_cluster_sweep_equal(monkeypatch, graph):
    """The impulse sweep by a cluster of 8 blocks per cloth (a variant the
    autotuner may pick) gives the same frames bit for bit, through contact."""
    cl = scene.config_batch(count=16)
    a = run(cl, "mixed", graph, 40)
    monkeypatch.setenv("CLOTHGPU_IMPULSE_CLUSTER", "8")
    b = run(cl, "mixed", graph, 40)
    assert same(a, b)
    assert sum(s["impulse_applied"] > 0 for fr in b[1] for s in fr) > 0


def test_autotune_leaves_frames_unchanged():
    """cs_autotune times candidate launch shapes on frames from the current state
    and restores it: the frames that follow equal those of an untuned context
    bit for bit, and a second context of the same shape takes the cached result."""
    from cloth_sim_self_collision_gb300 import build
    build.build()
    from cloth_sim_self_collision_gb300.context import ClothContext
    cl = scene.config_batch(count=12)
    out = []
    tunes = []
    for tune in (True, False, True):
        ctx = ClothContext(0, "mixed")
        try:
            ids = [ctx.add_cloth(c) for c in cl]
            ctx.step(28)
            if tune:
                tunes.append(ctx.autotune(2))
            ctx.step(4)
            out.append([ctx.get_state(i) for i in ids])
        finally:
            ctx.close()
    for a, b in ((out[0], out[1]), (out[2], out[1])):
        for (xa, va), (xb, vb) in zip(a, b):
            assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    t0, t1 = tunes
    print("autotune:", t0, t1)
    assert t0["cached"] == 0 and t0["candidates"] >= 3 and t0["frame_ms"] > 0
    assert t1["cached"] == 1 and t1["mx_blocks_per_sm"] == t0["mx_blocks_per_sm"]
    assert t0["mx_blocks_per_sm"] in (4, 5, 6) and t0["graph_grid_per_sm"] in (4, 8, 16)
    assert t0["narrow_regs"] in (0, 128) and t0["impulse_cluster"] in (1, 8)
