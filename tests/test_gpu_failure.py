"""Failure detection on the GPU without a GPU fault: the persistent solver's
grid barrier waits are bounded by the device clock.  A test hook keeps block 0
from arriving (CLOTHGPU_BAR_HOLD), so every wait runs out after a short limit
(CLOTHGPU_BAR_TIMEOUT_NS); the kernel flags it, every block leaves, and the
frame fails with CS_ERR_CUDA on the host, in host-driven and in graph frames.
The process's CUDA context stays usable: a context without the hook steps the
same cloths afterwards and matches a run that never saw the failure."""
import numpy as np
import pytest

from cloth_sim_self_collision_gb300 import scene

pytestmark = pytest.mark.gpu


def make(graph):
    from cloth_sim_self_collision_gb300 import build
    build.build()
    from cloth_sim_self_collision_gb300.context import ClothContext
    ctx = ClothContext(0, "mixed")
    ctx.frame_mode(graph)
    ids = [ctx.add_cloth(c) for c in scene.config_batch(count=6)]
    return ctx, ids


@pytest.mark.parametrize("graph", [False, True])
def test_barrier_time_out_fails_the_frame(monkeypatch, graph):
    from cloth_sim_self_collision_gb300 import _native as N
    monkeypatch.setenv("CLOTHGPU_BAR_HOLD", "1")
    monkeypatch.setenv("CLOTHGPU_BAR_TIMEOUT_NS", "20000000")  # 20 ms
    ctx, ids = make(graph)
    try:
        with pytest.raises(N.CsError) as e:
            ctx.step(1)
        assert e.value.code == N.CS_ERR_CUDA
        assert "grid barrier" in str(e.value)
    finally:
        ctx.close()
    monkeypatch.delenv("CLOTHGPU_BAR_HOLD")
    monkeypatch.delenv("CLOTHGPU_BAR_TIMEOUT_NS")
    out = []
    for _ in range(2):
        ctx, ids = make(graph)
        try:
            ctx.step(3)
            out.append([ctx.get_state(i) for i in ids])
        finally:
            ctx.close()
    for (xa, va), (xb, vb) in zip(*out):
        assert np.all(np.isfinite(xa)) and np.array_equal(xa, xb) and np.array_equal(va, vb)
