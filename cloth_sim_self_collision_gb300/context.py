"""Host-side Python API over the C ABI.

``ClothContext`` owns one device context; cloths are added from
``scene.Cloth`` descriptions and advanced together with ``step``.  The stage
methods mirror the reference's functions one to one (StepTime_InternalDynamics*,
GetIntermidiateVelocityContactResolved, UpdateIntermidiateVelocity, the BVH
and contact routines, the sparse solvers) on numpy arrays, with the same
argument meaning and in-place semantics as the reference.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N


class ClothContext:
    """A device context holding any number of cloths in one arena."""

    def __init__(self, device: int = 0, precision: str = "fp64"):
        self.L = N.load()
        h = ctypes.c_void_p()
        prec = {"fp64": N.CS_PREC_FP64, "mixed": N.CS_PREC_MIXED}[precision]
        rc = self.L.cs_create(device, prec, ctypes.byref(h))
        if rc != N.CS_OK:
            raise N.CsError(rc, "cs_create failed (no usable CUDA device?)")
        self.h = h
        self.np = {}

    def close(self):
        if self.h:
            self.L.cs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc != N.CS_OK:
            raise N.CsError(rc, self.L.cs_last_error(self.h).decode())

    # ---- cloths ---------------------------------------------------------------
    def add_cloth(self, cloth) -> int:
        X0 = np.ascontiguousarray(cloth.X0, np.float64)
        bc = np.ascontiguousarray(cloth.bc, np.int32)
        tri = np.ascontiguousarray(cloth.tri, np.int32)
        quad = np.ascontiguousarray(cloth.quad, np.int32)
        prm = N.CsParams.from_params(cloth.params)
        cid = ctypes.c_int()
        self._ck(self.L.cs_add_cloth(self.h, X0.size // 3, N.dp(X0), N.ip(bc), tri.size // 3, N.ip(tri),
                                     quad.size // 4, N.ip(quad), ctypes.byref(prm), ctypes.byref(cid)))
        self.np[cid.value] = X0.size // 3
        return cid.value

    def remove_cloth(self, cid: int):
        self._ck(self.L.cs_remove_cloth(self.h, cid))
        del self.np[cid]

    def set_params(self, cid: int, params):
        prm = N.CsParams.from_params(params)
        self._ck(self.L.cs_set_params(self.h, cid, ctypes.byref(prm)))

    def set_state(self, cid: int, x=None, v=None):
        xa = None if x is None else np.ascontiguousarray(x, np.float64)
        va = None if v is None else np.ascontiguousarray(v, np.float64)
        self._ck(self.L.cs_set_state(self.h, cid, None if xa is None else N.dp(xa),
                                     None if va is None else N.dp(va)))

    def get_state(self, cid: int):
        n = 3 * self.np[cid]
        x = np.empty(n)
        v = np.empty(n)
        self._ck(self.L.cs_get_state(self.h, cid, N.dp(x), N.dp(v)))
        return x, v

    def stats(self, cid: int) -> dict:
        st = N.CsStats()
        self._ck(self.L.cs_get_stats(self.h, cid, ctypes.byref(st)))
        return st.as_dict()

    def step(self, nsteps: int = 1):
        """StepTime of every cloth, nsteps times (self_contact_sparse/main.cpp:213-263)."""
        self._ck(self.L.cs_step(self.h, nsteps))

    def synchronize(self):
        self._ck(self.L.cs_synchronize(self.h))

    def launch_count(self) -> int:
        return int(self.L.cs_launch_count(self.h))

    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return int(self.L.cs_stream(self.h) or 0)

    def num_vertices(self) -> int:
        return int(self.L.cs_num_vertices(self.h))

    def set_states(self, x=None, v=None):
        """States of all cloths, back to back in the order they were added."""
        self._ck(self.L.cs_set_states(self.h, None if x is None else N.dp(x), None if v is None else N.dp(v)))

    def get_states(self, x, v):
        self._ck(self.L.cs_get_states(self.h, None if x is None else N.dp(x), None if v is None else N.dp(v)))

    def profile(self, enable: bool):
        self._ck(self.L.cs_profile(self.h, 1 if enable else 0))

    def profile_bytes(self):
        """(FP32 SpMV bytes, FP64 SpMV bytes) since profiling was enabled."""
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        self._ck(self.L.cs_profile_bytes(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def profile_read(self, kernel: str):
        ms = ctypes.c_double()
        n = ctypes.c_longlong()
        self._ck(self.L.cs_profile_read(self.h, kernel.encode(), ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def autotune(self, frames: int = 2) -> dict:
        """Launch shapes timed on `frames` frames from the current state (which is
        restored); the fastest are kept and cached per arena shape."""
        r = N.CsTuneResult()
        self._ck(self.L.cs_autotune(self.h, frames, ctypes.byref(r)))
        return r.as_dict()

    def frame_mode(self, graph: bool):
        """Frames as one captured CUDA graph each (True, the default) or host-driven."""
        self._ck(self.L.cs_set_frame_mode(self.h, 1 if graph else 0))

    def frame_counts(self) -> dict:
        """Graph frames, host-driven frames, graph captures, graph frames re-run host-driven."""
        v = [ctypes.c_longlong() for _ in range(4)]
        self._ck(self.L.cs_frame_counts(self.h, *[ctypes.byref(x) for x in v]))
        d = dict(zip(("graph_frames", "host_frames", "captures", "overflows"), (x.value for x in v)))
        r = (ctypes.c_longlong * 4)()
        self._ck(self.L.cs_frame_overflows(self.h, r))
        d["overflow_reasons"] = dict(zip(("sort", "zone", "buffers", "solver"), r))
        return d

    def log_contacts(self, enable: bool = True):
        """Record, per detection of each cloth's next contact resolution, (kind,
        count, digest of the ordered contact list)."""
        self._ck(self.L.cs_contact_log(self.h, 1 if enable else 0))

    def contact_log(self, cid: int):
        """The detections of the cloth's last resolution: a list of (ccd, count, digest)."""
        n = ctypes.c_int()
        self._ck(self.L.cs_contact_log_read(self.h, cid, None, None, None, 0, ctypes.byref(n)))
        m = max(n.value, 1)
        k = np.zeros(m, np.int32)
        c = np.zeros(m, np.int32)
        d = np.zeros(m, np.uint64)
        self._ck(self.L.cs_contact_log_read(self.h, cid, N.ip(k), N.ip(c),
                                            d.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong)), m,
                                            ctypes.byref(n)))
        return [(int(k[i]), int(c[i]), int(d[i])) for i in range(n.value)]

    # ---- stages (host arrays in / out) -------------------------------------------
    def implicit(self, cid, x, v):
        """StepTime_InternalDynamicsILU / StepTime_InternalDynamics (solve_internal_sparse.h:185-326)."""
        x = np.array(x, np.float64)
        v = np.array(v, np.float64)
        st = N.CsStats()
        self._ck(self.L.cs_implicit_step(self.h, cid, N.dp(x), N.dp(v), ctypes.byref(st)))
        return x, v, st.as_dict()

    def resolve(self, cid, x1, v):
        """GetIntermidiateVelocityContactResolved (self_collision_cloth.cpp:355-456)."""
        x1 = np.ascontiguousarray(x1, np.float64)
        v = np.array(v, np.float64)
        st = N.CsStats()
        self._ck(self.L.cs_resolve_contacts(self.h, cid, N.dp(x1), N.dp(v), ctypes.byref(st)))
        return v, st.as_dict()

    def update_velocity(self, cid, x, v):
        """UpdateIntermidiateVelocity (solve_internal_sparse.h:329-369)."""
        x = np.ascontiguousarray(x, np.float64)
        v = np.array(v, np.float64)
        self._ck(self.L.cs_update_velocity(self.h, cid, N.dp(x), N.dp(v)))
        return v

    def vertex_normals(self, cid: int = -1, x=None):
        """MakeNormal (self_contact_sparse/main.cpp:183-211): unit vertex normals of
        cloth cid at positions x (default: its state), or of every cloth (cid = -1)."""
        if cid < 0:
            out = np.empty(3 * self.num_vertices())
            self._ck(self.L.cs_vertex_normals(self.h, -1, None, N.dp(out)))
            return out
        out = np.empty(3 * self.np[cid])
        xa = None if x is None else np.ascontiguousarray(x, np.float64)
        self._ck(self.L.cs_vertex_normals(self.h, cid, None if xa is None else N.dp(xa), N.dp(out)))
        return out

    def pattern(self, cid):
        """Block pattern of the cloth's matrix (CMatrixSquareSparse::SetPattern,
        matrix_square_sparse.cpp:140-165): row pointer and sorted columns."""
        nb = ctypes.c_int()
        self._ck(self.L.cs_pattern(self.h, cid, ctypes.byref(nb), None, None))
        rp = np.zeros(self.np[cid] + 1, np.int32)
        ci = np.zeros(nb.value, np.int32)
        self._ck(self.L.cs_pattern(self.h, cid, None, N.ip(rp), N.ip(ci)))
        return rp, ci

    def assemble(self, cid, x, v):
        """Implicit system at (x, v): AddWdWddW_Cloth / _Contact / Mearge /
        SetBoundaryCondition (solve_internal_sparse.h:19-183, matrix_square_sparse.cpp:88-302).
        Returns the diagonal and off-diagonal blocks and the right-hand side."""
        nb = ctypes.c_int()
        self._ck(self.L.cs_pattern(self.h, cid, ctypes.byref(nb), None, None))
        n = self.np[cid]
        vd = np.zeros(9 * n)
        vc = np.zeros(9 * nb.value)
        b = np.zeros(3 * n)
        self._ck(self.L.cs_assemble(self.h, cid, N.dp(np.ascontiguousarray(x, np.float64)),
                                    N.dp(np.ascontiguousarray(v, np.float64)), N.dp(vd), N.dp(vc), N.dp(b)))
        return vd, vc, b

    def ilu(self, cid):
        """Block ILU(0) of the last assembled matrix: SetValueILU and DoILUDecomp
        (ilu_sparse.cpp:352-624).  Returns the factor blocks and the singular-pivot count."""
        nb = ctypes.c_int()
        self._ck(self.L.cs_pattern(self.h, cid, ctypes.byref(nb), None, None))
        fd = np.zeros(9 * self.np[cid])
        fc = np.zeros(9 * nb.value)
        ns = ctypes.c_int()
        self._ck(self.L.cs_ilu_factor(self.h, cid, N.dp(fd), N.dp(fc), ctypes.byref(ns)))
        return fd, fc, ns.value

    def pcg(self, cid, b, tol, maxit):
        """Solve_PCG with the ILU(0) factor (ilu_sparse.cpp:628-709)."""
        x = np.zeros(3 * self.np[cid])
        conv = ctypes.c_double()
        it = ctypes.c_int()
        self._ck(self.L.cs_solve_pcg(self.h, cid, N.dp(np.ascontiguousarray(b, np.float64)), tol, maxit, N.dp(x),
                                     ctypes.byref(conv), ctypes.byref(it)))
        return x, conv.value, it.value

    def cg(self, cid, b, tol, maxit):
        """Solve_CG, unpreconditioned (matrix_square_sparse.cpp:338-406)."""
        x = np.zeros(3 * self.np[cid])
        conv = ctypes.c_double()
        it = ctypes.c_int()
        self._ck(self.L.cs_solve_cg(self.h, cid, N.dp(np.ascontiguousarray(b, np.float64)), tol, maxit, N.dp(x),
                                    ctypes.byref(conv), ctypes.byref(it)))
        return x, conv.value, it.value

    def spmv(self, cid, x):
        """y = A x with the last assembled matrix (CMatrixSquareSparse::MatVec,
        matrix_square_sparse.cpp:167-270)."""
        y = np.zeros(3 * self.np[cid])
        self._ck(self.L.cs_spmv(self.h, cid, N.dp(np.ascontiguousarray(x, np.float64)), N.dp(y)))
        return y

    def bvh_nodes(self, cid):
        """BVH nodes (parent, child 0, child 1; child 1 = -1 at a leaf) as
        MakeBVHTopology_TopDown builds them (bvh_aabb.cpp:109-313)."""
        nn = ctypes.c_int()
        self._ck(self.L.cs_bvh_nodes(self.h, cid, ctypes.byref(nn), None))
        out = np.zeros(3 * nn.value, np.int32)
        self._ck(self.L.cs_bvh_nodes(self.h, cid, None, N.ip(out)))
        return out.reshape(-1, 3)

    def _nnode(self, cid):
        nn = ctypes.c_int()
        self._ck(self.L.cs_bvh_nodes(self.h, cid, ctypes.byref(nn), None))
        return nn.value

    def refit_prx(self, cid, x, delta):
        """Node boxes for proximity (BuildBoundingBoxChild_Prx, bvh_aabb.cpp:23-61)."""
        out = np.zeros(7 * self._nnode(cid))
        self._ck(self.L.cs_refit_prx(self.h, cid, N.dp(np.ascontiguousarray(x, np.float64)), delta, N.dp(out)))
        return out.reshape(-1, 7)

    def refit_ccd(self, cid, x, v, dt):
        """Swept node boxes (BuildBoundingBoxChild_CCD, bvh_aabb.cpp:64-106)."""
        out = np.zeros(7 * self._nnode(cid))
        self._ck(self.L.cs_refit_ccd(self.h, cid, N.dp(np.ascontiguousarray(x, np.float64)),
                                     N.dp(np.ascontiguousarray(v, np.float64)), dt, N.dp(out)))
        return out.reshape(-1, 7)

    def _contacts(self, fn, *args, cap=1 << 16):
        while True:
            out = np.zeros(5 * cap, np.int32)
            n = ctypes.c_int()
            rc = fn(*args, N.ip(out), cap, ctypes.byref(n))
            if rc == N.CS_ERR_CAPACITY:
                cap = n.value
                continue
            self._ck(rc)
            return out[: 5 * n.value].reshape(-1, 5)

    def contacts_prx(self, cid, x, delta):
        """Proximity contact set in std::set order (GetContactElement_Proximity,
        bvh_aabb.cpp:441-557): rows (i0, i1, i2, i3, is_fv)."""
        xa = np.ascontiguousarray(x, np.float64)
        return self._contacts(self.L.cs_contacts_prx, self.h, cid, N.dp(xa), delta)

    def contacts_ccd(self, cid, x, v, dt, delta):
        """CCD contact set in std::set order (GetContactElement_CCD, bvh_aabb.cpp:797-923)."""
        xa = np.ascontiguousarray(x, np.float64)
        va = np.ascontiguousarray(v, np.float64)
        return self._contacts(self.L.cs_contacts_ccd, self.h, cid, N.dp(xa), N.dp(va), dt, delta)

    def impulse_prx(self, cid, x, v, ce):
        """SelfCollisionImpulse_Proximity over the contacts ce (self_collision_cloth.cpp:20-112)."""
        v = np.array(v, np.float64)
        ce = np.ascontiguousarray(ce, np.int32)
        self._ck(self.L.cs_impulse_prx(self.h, cid, N.dp(np.ascontiguousarray(x, np.float64)), N.dp(v), N.ip(ce),
                                       ce.shape[0]))
        return v

    def impulse_ccd(self, cid, x, v, ce):
        """SelfCollisionImpulse_CCD over the contacts ce (self_collision_cloth.cpp:116-212)."""
        v = np.array(v, np.float64)
        ce = np.ascontiguousarray(ce, np.int32)
        self._ck(self.L.cs_impulse_ccd(self.h, cid, N.dp(np.ascontiguousarray(x, np.float64)), N.dp(v), N.ip(ce),
                                       ce.shape[0]))
        return v

    def riz_reset(self, cid):
        """Empties the cloth's rigid impact zones."""
        self._ck(self.L.cs_riz_reset(self.h, cid))

    def riz_add(self, cid, ce):
        """MakeRigidImpactZone with the contacts ce (self_collision_cloth.cpp:220-274)."""
        ce = np.ascontiguousarray(ce, np.int32)
        self._ck(self.L.cs_riz_add(self.h, cid, N.ip(ce), ce.shape[0]))

    def riz_zones(self, cid):
        """Zone of every vertex (-1 outside all zones) and the number of zones."""
        z = np.zeros(self.np[cid], np.int32)
        nz = ctypes.c_int()
        self._ck(self.L.cs_riz_zones(self.h, cid, N.ip(z), ctypes.byref(nz)))
        return z, nz.value

    def riz_apply(self, cid, x, v, v0):
        """ApplyRigidImpactZone (self_collision_cloth.cpp:298-348)."""
        v = np.array(v, np.float64)
        self._ck(self.L.cs_riz_apply(self.h, cid, N.dp(np.ascontiguousarray(x, np.float64)), N.dp(v),
                                     N.dp(np.ascontiguousarray(v0, np.float64))))
        return v

    # ---- element batches ---------------------------------------------------------------
    def element_cst(self, C, c, lam, myu):
        """WdWddW_CST per triangle (cloth_internal_physics.h:70-176)."""
        C = np.ascontiguousarray(C, np.float64).reshape(-1, 9)
        c = np.ascontiguousarray(c, np.float64).reshape(-1, 9)
        n = C.shape[0]
        W, dW, ddW = np.zeros(n), np.zeros((n, 9)), np.zeros((n, 81))
        self._ck(self.L.cs_element_cst(self.h, n, N.dp(C), N.dp(c), lam, myu, N.dp(W), N.dp(dW), N.dp(ddW)))
        return W, dW, ddW

    def element_bend(self, C, c, stiff):
        """WdWddW_Bend per stencil (cloth_internal_physics.h:180-238)."""
        C = np.ascontiguousarray(C, np.float64).reshape(-1, 12)
        c = np.ascontiguousarray(c, np.float64).reshape(-1, 12)
        n = C.shape[0]
        W, dW, ddW = np.zeros(n), np.zeros((n, 12)), np.zeros((n, 144))
        self._ck(self.L.cs_element_bend(self.h, n, N.dp(C), N.dp(c), stiff, N.dp(W), N.dp(dW), N.dp(ddW)))
        return W, dW, ddW

    def element_contact(self, c, params):
        """WdWddW_Contact per vertex with the cloth's obstacle (cloth_internal_physics.h:243-280)."""
        c = np.ascontiguousarray(c, np.float64).reshape(-1, 3)
        n = c.shape[0]
        W, dW, ddW = np.zeros(n), np.zeros((n, 3)), np.zeros((n, 9))
        prm = N.CsParams.from_params(params)
        self._ck(self.L.cs_element_contact(self.h, n, N.dp(c), ctypes.byref(prm), N.dp(W), N.dp(dW), N.dp(ddW)))
        return W, dW, ddW
