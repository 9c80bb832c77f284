"""Python mirror of the serving entry points (``cs_server_*`` of include/clothgpu.h).

A :class:`Server` owns one native worker thread and one device arena: scenes
submitted at any time are admitted by estimated device bytes, packed into the
next arena off the critical path, swapped in at a frame boundary, and advanced
together with every other resident scene, one frame of
``StepTime`` (self_contact_sparse/main.cpp:213-263) per loop.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N
from .scene import Cloth

_PREC = {"fp64": N.CS_PREC_FP64, "mixed": N.CS_PREC_MIXED}


class Server:
    def __init__(self, device: int = 0, precision: str = "mixed", hbm_budget_bytes: float = 150e9,
                 max_cloths: int = 0):
        self._L = N.load()
        cfg = N.CsServerConfig(device, _PREC[precision], float(hbm_budget_bytes), int(max_cloths))
        h = ctypes.c_void_p()
        code = self._L.cs_server_create(ctypes.byref(cfg), ctypes.byref(h))
        if code != N.CS_OK:
            raise N.CsError(code, "cs_server_create failed")
        self._h = h
        self._np = {}

    def _check(self, code: int, what: str):
        if code != N.CS_OK:
            msg = self._L.cs_server_last_error(self._h)
            raise N.CsError(code, f"{what}: {msg.decode() if msg else ''}")

    def submit(self, cloth: Cloth, nsteps: int, x: np.ndarray | None = None,
               v: np.ndarray | None = None) -> int:
        """Queues ``cloth`` for ``nsteps`` frames; returns the request id."""
        X0 = np.ascontiguousarray(cloth.X0, dtype=np.float64)
        tri = np.ascontiguousarray(cloth.tri, dtype=np.int32)
        quad = np.ascontiguousarray(cloth.quad, dtype=np.int32)
        bc = np.ascontiguousarray(cloth.bc, dtype=np.int32)
        xa = None if x is None else np.ascontiguousarray(x, dtype=np.float64)
        va = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        prm = N.CsParams.from_params(cloth.params)
        req = ctypes.c_int()
        self._check(self._L.cs_server_submit(
            self._h, cloth.np, N.dp(X0), N.ip(bc), cloth.nt, N.ip(tri), cloth.nq, N.ip(quad),
            None if xa is None else N.dp(xa), None if va is None else N.dp(va), ctypes.byref(prm),
            int(nsteps), ctypes.byref(req)), "cs_server_submit")
        self._np[req.value] = cloth.np
        return req.value

    def wait(self, req: int, timeout: float = -1.0):
        """Blocks until the request finishes; returns (x, v, info)."""
        n = self._np[req]
        x = np.empty(3 * n)
        v = np.empty(3 * n)
        info = N.CsRequestInfo()
        self._check(self._L.cs_server_wait(self._h, req, float(timeout), N.dp(x), N.dp(v), ctypes.byref(info)),
                    f"cs_server_wait({req})")
        return x, v, info.as_dict()

    def release(self, req: int):
        self._check(self._L.cs_server_release(self._h, req), "cs_server_release")

    def drain(self, timeout: float = -1.0):
        self._check(self._L.cs_server_drain(self._h, float(timeout)), "cs_server_drain")

    def stats(self) -> dict:
        st = N.CsServerStats()
        self._check(self._L.cs_server_get_stats(self._h, ctypes.byref(st)), "cs_server_get_stats")
        return st.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            self._L.cs_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()


def scene_device_bytes(cloth: Cloth) -> int:
    """The server's admission estimate of a scene's device bytes."""
    L = N.load()
    X0 = np.ascontiguousarray(cloth.X0, dtype=np.float64)
    tri = np.ascontiguousarray(cloth.tri, dtype=np.int32)
    quad = np.ascontiguousarray(cloth.quad, dtype=np.int32)
    prm = N.CsParams.from_params(cloth.params)
    return int(L.cs_scene_device_bytes(cloth.np, N.dp(X0), cloth.nt, N.ip(tri), cloth.nq, N.ip(quad),
                                       ctypes.byref(prm)))
