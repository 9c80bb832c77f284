"""Proximity contact sets near the decision boundaries of the narrow phase.

The FP32 prefilters in front of the FP64 tests (outward-rounded boxes,
directed-rounding slab bounds, and the edge-edge closest-point / line-distance
filter with its error bounds) may only reject pairs that the reference's FP64
test rejects.  Crumpled sheets put many edge pairs near every threshold (the
clearance, the segment ends, near-parallel edges); the contact lists must equal
the oracle's bit for bit."""
import numpy as np
import pytest

from cloth_sim_self_collision_gb300 import scene
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from cloth_sim_self_collision_gb300 import build
    build.build()
    from cloth_sim_self_collision_gb300.context import ClothContext
    c = ClothContext()
    yield c
    c.close()


def crumpled(c, seed, amp_xy, amp_z):
    """The sheet's rest shape with a smooth fold plus random jitter: layers and
    neighbours at distances around the clearance."""
    rng = np.random.default_rng(seed)
    X = c.X0.reshape(-1, 3).copy()
    X[:, 2] += 0.05 * np.sin(7.0 * X[:, 0]) * np.cos(5.0 * X[:, 1])
    X[:, :2] += rng.uniform(-amp_xy, amp_xy, (len(X), 2))
    X[:, 2] += rng.uniform(-amp_z, amp_z, len(X))
    return X.reshape(-1)


@pytest.mark.parametrize("seed", range(6))
def test_prx_contacts_crumpled(ctx, oracle_port, seed):
    c = scene.square_cloth(31, 0.5, 0.4, sphere_radius=0.2, clearance=0.01, seed=20 + seed,
                           solver_kind=scene.SOLVER_CG, tol=1e-6, maxit=1000)
    cid = ctx.add_cloth(c)
    orc = O.OracleCloth(oracle_port, c)
    x = crumpled(c, seed, amp_xy=0.004 * (1 + seed), amp_z=0.006 * (1 + seed % 3))
    total = 0
    for delta in (0.005, 0.01, 0.02, 0.04):
        a = ctx.contacts_prx(cid, x, delta)
        b = orc.contacts_prx(x, delta)
        assert np.array_equal(a, b), (seed, delta, len(a), len(b))
        total += len(b)
    ctx.remove_cloth(cid)
    orc.close()
    assert total > 0


def test_prx_contacts_fold_probe_scaled(ctx, oracle_port):
    """The folded sheet's probe state squeezed toward its centroid: layers cross
    the clearance one after another."""
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    arr = dict(np.load(os.path.join(here, "golden", "fold_31.npz")))
    c = scene.square_cloth(31, 1.0, 0.4, sphere_radius=0.2, clearance=0.01, seed=11,
                           solver_kind=scene.SOLVER_CG, tol=1.0e-6, maxit=1000)
    cid = ctx.add_cloth(c)
    orc = O.OracleCloth(oracle_port, c)
    X = arr["probe_x"].reshape(-1, 3)
    g = X.mean(axis=0)
    for s in (1.0, 0.9, 0.75, 0.6, 0.5):
        x = (g + s * (X - g)).reshape(-1)
        a = ctx.contacts_prx(cid, x, 0.01)
        b = orc.contacts_prx(x, 0.01)
        assert np.array_equal(a, b), (s, len(a), len(b))
    ctx.remove_cloth(cid)
    orc.close()


@pytest.mark.parametrize("seed", range(5))
def test_ccd_contacts_crumpled(ctx, oracle_port, seed):
    """CCD contact sets on crumpled sheets moving with random velocities of
    several scales: coplanarity times cross [0, 1] at many pairs, which the FP32
    certificates in front of the FP64 tests (the no-root certificate of the
    coplanarity cubic for both kinds, the face-vertex sign block) must never
    reject.  The batch's own contact frames are covered by the contact logs of
    tests/test_gpu_mixed_batch.py."""
    c = scene.square_cloth(31, 0.5, 0.4, sphere_radius=0.2, clearance=0.01, seed=40 + seed,
                           solver_kind=scene.SOLVER_CG, tol=1e-6, maxit=1000)
    cid = ctx.add_cloth(c)
    orc = O.OracleCloth(oracle_port, c)
    rng = np.random.default_rng(100 + seed)
    x = crumpled(c, seed, amp_xy=0.003 * (1 + seed), amp_z=0.005 * (1 + seed % 3))
    total = 0
    for scale in (1e-4, 1e-3, 0.05, 0.3, 1.0, 3.0):
        v = rng.normal(0.0, scale, x.size)
        v[2::3] -= 2.0  # a common downward drift, as when falling
        a = ctx.contacts_ccd(cid, x, v, c.params.dt, c.params.contact_clearance)
        b = orc.contacts_ccd(x, v, c.params.dt, c.params.contact_clearance)
        assert np.array_equal(a, b), (seed, scale, len(a), len(b))
        total += len(b)
    ctx.remove_cloth(cid)
    orc.close()
    assert total > 0


@pytest.mark.parametrize("seed", range(3))
def test_ccd_contacts_flat_sheet_crossing(ctx, oracle_port, seed):
    """A flat sheet (only its 1e-4 jitter off the plane) whose vertices move
    across their neighbours' face planes by about the jitter: signed heights and
    coplanarity cubics near zero at nearly every face-vertex pair."""
    c = scene.square_cloth(41, 0.5, 0.4, sphere_radius=0.2, clearance=0.01, seed=60 + seed,
                           solver_kind=scene.SOLVER_CG, tol=1e-6, maxit=1000)
    cid = ctx.add_cloth(c)
    orc = O.OracleCloth(oracle_port, c)
    rng = np.random.default_rng(200 + seed)
    x = c.X0.copy()
    total = 0
    for scale in (1e-3, 5e-3, 2e-2):
        v = np.zeros_like(x)
        v[2::3] = rng.normal(0.0, scale, x.size // 3) - 1.0
        v[0::3] = rng.normal(0.0, 0.1 * scale, x.size // 3)
        a = ctx.contacts_ccd(cid, x, v, c.params.dt, c.params.contact_clearance)
        b = orc.contacts_ccd(x, v, c.params.dt, c.params.contact_clearance)
        assert np.array_equal(a, b), (seed, scale, len(a), len(b))
        total += len(b)
    ctx.remove_cloth(cid)
    orc.close()
