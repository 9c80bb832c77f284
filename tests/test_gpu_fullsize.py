"""Parity at the single-cloth configurations' full sizes (101x101 sheet, 256x256
sheet): one frame from the initial state.  With serial inner products the
device frame equals the oracle's bit for bit (positions, velocities, contact
counts); the mixed-precision frame meets the reference's solver criterion on the
oracle's FP64 system and finds the same contacts."""
import numpy as np
import pytest

from cloth_sim_self_collision_gb300 import scene
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cloth_sim_self_collision_gb300 import build
    build.build()


def _exact(c):
    c.params.flags = 1  # CS_FLAG_EXACT_DOTS
    return c


@pytest.mark.parametrize("name", ["single_101", "single_256"])
def test_first_frame_bit_exact(oracle_port, name):
    from cloth_sim_self_collision_gb300.context import ClothContext
    c = _exact(scene.config_single_101() if name == "single_101" else scene.config_single_256())
    orc = O.OracleCloth(oracle_port, c)
    so = orc.step(1)[0]
    ctx = ClothContext(0, "fp64")
    cid = ctx.add_cloth(c)
    ctx.step(1)
    x, v = ctx.get_state(cid)
    sg = ctx.stats(cid)
    ctx.close()
    assert sg["n_prx"] == so["n_prx"] and sg["n_ccd"][:5] == so["n_ccd"][:5]
    assert sg["solver_iterations"] == so["solver_iterations"]
    assert np.array_equal(x, orc.x) and np.array_equal(v, orc.v)


@pytest.mark.parametrize("name", ["single_101", "single_256"])
def test_first_frame_mixed(oracle_port, name):
    from cloth_sim_self_collision_gb300.context import ClothContext
    from tests.test_gpu_parity import residual_ratio
    c = scene.config_single_101() if name == "single_101" else scene.config_single_256()
    orc = O.OracleCloth(oracle_port, c)
    x0, v0 = orc.x.copy(), orc.v.copy()
    vd, vc, b = orc.assemble(x0, v0)
    rp, ci = orc.pattern()
    ctx = ClothContext(0, "mixed")
    cid = ctx.add_cloth(c)
    xa, va, sa = ctx.implicit(cid, x0, v0)
    assert residual_ratio(vd, vc, rp, ci, b, xa - x0) < c.params.tol
    # contact detection on identical inputs: the same set
    assert np.array_equal(ctx.contacts_prx(cid, x0, c.params.contact_clearance),
                          orc.contacts_prx(x0, c.params.contact_clearance))
    ctx.close()
