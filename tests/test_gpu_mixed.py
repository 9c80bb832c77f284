"""Mixed-precision solve (CS_PREC_MIXED): FP32 block-Jacobi CG inside FP64
iterative refinement.  Bounds, per implicit step along the oracle's trajectory:

* the increment meets the reference's criterion (relative residual below the
  tolerance) on the FP64 system the oracle assembles;
* against the exact solution of that system (the oracle solved to 1e-12), the
  mixed path's position error is no larger than the reference's own error at
  its tolerance, and below MIXED_RTOL relative."""
import numpy as np
import pytest

from cloth_sim_self_collision_gb300 import scene
from oracle import oracle as O
from tests.test_gpu_parity import fold_scene, residual_ratio

pytestmark = pytest.mark.gpu

MIXED_RTOL = 1e-6


@pytest.fixture(scope="module")
def mctx():
    from cloth_sim_self_collision_gb300 import build
    build.build()
    from cloth_sim_self_collision_gb300.context import ClothContext
    c = ClothContext(0, "mixed")
    yield c
    c.close()


@pytest.mark.parametrize("name", ["small_21", "fold_31", "batch_61"])
def test_mixed_implicit_accuracy(mctx, oracle_port, name):
    if name == "small_21":
        c = scene.config_small()
    elif name == "fold_31":
        c = fold_scene()
    else:
        c = scene.square_cloth(61, 1.0, 0.6, sphere_radius=0.25, seed=5, solver_kind=scene.SOLVER_CG,
                               tol=1e-6, maxit=1000)
    cid = mctx.add_cloth(c)
    orc = O.OracleCloth(oracle_port, c)
    tight = O.OracleCloth(oracle_port, c)
    tp = scene.Params(**dict(c.params.__dict__))
    tp.solver_kind, tp.tol, tp.maxit = scene.SOLVER_CG, 1e-12, 50000
    tight.set_params(tp)
    rp, ci = orc.pattern()
    worst = 0.0
    for f in range(0, 80, 8):
        x0 = orc.x.copy()
        vd, vc, b = orc.assemble(orc.x, orc.v)
        xa, va, sa = mctx.implicit(cid, orc.x, orc.v)
        xb, vb, sb = orc.implicit(orc.x, orc.v)
        xt, vt, st = tight.implicit(orc.x, orc.v)
        ra = residual_ratio(vd, vc, rp, ci, b, xa - x0)
        assert ra < c.params.tol, (name, f, ra)
        scale = max(1.0, np.abs(xt).max())
        err_mixed = np.abs(xa - xt).max() / scale
        err_ref = np.abs(xb - xt).max() / scale
        worst = max(worst, err_mixed)
        assert err_mixed <= max(err_ref, 1e-9), (name, f, err_mixed, err_ref)
        assert err_mixed <= MIXED_RTOL, (name, f, err_mixed)
        orc.step(8)
    print(f"{name}: worst position error of the mixed implicit step vs the exact solve {worst:.2e}")
    mctx.remove_cloth(cid)


def test_mixed_frames_contacts(mctx, oracle_port):
    """Whole frames of the folding sheet from oracle states, against the
    oracle's frame with the implicit system solved to 1e-12 (the reference at
    its own tolerance of 1e-6 is up to 2.4e-6 away from that frame here): the
    same ordered contact list in every detection (contact log), positions
    within MIXED_RTOL, and velocities within the same bound as the position
    change they make over the frame (|dv| dt)."""
    import dataclasses
    c = fold_scene()
    cid = mctx.add_cloth(c)
    orc = O.OracleCloth(oracle_port, c)
    tight = dataclasses.replace(c.params, tol=1e-12, maxit=50000)
    mctx.log_contacts(True)
    frame = 0
    try:
        for f in [30, 34, 38, 45, 60, 90]:
            orc.step(f - frame)
            frame = f
            mctx.set_state(cid, orc.x, orc.v)
            nxt = O.OracleCloth(oracle_port, c)
            nxt.set_params(tight)
            nxt.x, nxt.v = orc.x.copy(), orc.v.copy()
            nxt.log_contacts(True)
            nxt.step(1)
            mctx.step(1)
            xa, va = mctx.get_state(cid)
            scale = max(1.0, np.abs(nxt.x).max())
            ex = np.abs(xa - nxt.x).max() / scale
            ev = np.abs(va - nxt.v).max() * c.params.dt / scale
            la, lb = mctx.contact_log(cid), nxt.contact_log()
            print(f"frame {f}: x {ex:.2e} |dv| dt {ev:.2e} detections {len(la)} contacts {sum(n for _, n, _ in la)}")
            assert la == lb, (f, [(k, n) for k, n, _ in la], [(k, n) for k, n, _ in lb])
            assert ex <= MIXED_RTOL and ev <= MIXED_RTOL, (f, ex, ev)
            nxt.close()
    finally:
        mctx.log_contacts(False)
        mctx.remove_cloth(cid)


def test_mixed_batch_runs(mctx):
    cl = scene.config_batch(count=16)
    ids = [mctx.add_cloth(c) for c in cl]
    mctx.step(4)
    for i in ids:
        x, v = mctx.get_state(i)
        assert np.all(np.isfinite(x)) and np.all(np.isfinite(v))
        st = mctx.stats(i)
        assert st["solver_conv"] < 1e-6
    for i in ids:
        mctx.remove_cloth(i)


def _small_sheets(n):
    rng = np.random.default_rng(11)
    out = []
    for i in range(n):
        side = int(rng.integers(4, 9))
        r = float(rng.uniform(0.05, 0.2))
        out.append(scene.square_cloth(side, 0.1 * (side - 1), r + float(rng.uniform(0.02, 0.1)),
                                      sphere_radius=r, seed=i,
                                      rotation=float(rng.uniform(0, 6.28)), solver_kind=scene.SOLVER_CG,
                                      tol=1e-6, maxit=1000))
    return out


def test_mixed_static_cut_same_result_alone():
    """More than 2048 cloths: the persistent solver keeps a static cut of the
    slices over its blocks (below that it re-cuts the still-iterating cloths'
    slices).  Either way each cloth's totals are its own fixed-order sums, so a
    cloth steps bit-identically in the 2100-cloth arena and alone."""
    from cloth_sim_self_collision_gb300.context import ClothContext
    cl = _small_sheets(2100)
    big = ClothContext(0, "mixed")
    try:
        ids = [big.add_cloth(c) for c in cl]
        big.step(3)
        many = {i: big.get_state(ids[i]) for i in (0, 777, 2099)}
        for i in (0, 777, 2099):
            assert big.stats(ids[i])["solver_conv"] < 1e-6
    finally:
        big.close()
    for i in (0, 777, 2099):
        one = ClothContext(0, "mixed")
        try:
            cid = one.add_cloth(cl[i])
            one.step(3)
            x, v = one.get_state(cid)
        finally:
            one.close()
        assert np.array_equal(x, many[i][0]) and np.array_equal(v, many[i][1]), i
