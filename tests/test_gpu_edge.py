"""Edge cases of the context on the GPU: an empty arena (no cloths, and after
the last cloth is removed) steps, profiles and autotunes without error, for both
precisions and frame modes; a cloth added afterwards steps like one in a fresh
context."""
import numpy as np
import pytest

from cloth_sim_self_collision_gb300 import scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("graph", [True, False])
def test_empty_arena(prec, graph):
    from cloth_sim_self_collision_gb300 import build
    build.build()
    from cloth_sim_self_collision_gb300.context import ClothContext
    c = scene.config_batch(count=2)[1]
    ctx = ClothContext(0, prec)
    try:
        ctx.frame_mode(graph)
        ctx.profile(True)
        ctx.step(2)
        ctx.profile(False)
        i = ctx.add_cloth(c)
        ctx.remove_cloth(i)
        ctx.step(1)
        j = ctx.add_cloth(c)
        ctx.step(3)
        got = ctx.get_state(j)
    finally:
        ctx.close()
    ref = ClothContext(0, prec)
    try:
        ref.frame_mode(graph)
        k = ref.add_cloth(c)
        ref.step(3)
        want = ref.get_state(k)
    finally:
        ref.close()
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
