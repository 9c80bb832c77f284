"""ctypes bindings of the oracle -- TEST INFRASTRUCTURE ONLY.

Two libraries share one C interface (cloth_oracle.h):

* ``port``: the plain-C restatement, oracle/_build/libclothoracle.so
* ``ref``:  the reference's own sources compiled in place with the headless
            driver, oracle/_ref/libclothref.so (only where the reference
            sources exist at build time)

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module; the CUDA library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libclothoracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libclothref.so")
# the reference checkout: CLOTH_REFERENCE_DIR, else beside this repository's checkout
REF_SRC = os.environ.get("CLOTH_REFERENCE_DIR", os.path.normpath(os.path.join(HERE, "..", "..", "reference")))


class CoParams(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double), ("lam", ctypes.c_double), ("myu", ctypes.c_double),
        ("stiff_bend", ctypes.c_double), ("gravity", ctypes.c_double * 3),
        ("mass_point", ctypes.c_double), ("stiff_contact", ctypes.c_double),
        ("contact_clearance", ctypes.c_double), ("obs_center", ctypes.c_double * 3),
        ("obs_radius", ctypes.c_double), ("tol", ctypes.c_double),
        ("obstacle_kind", ctypes.c_int), ("solver_kind", ctypes.c_int),
        ("maxit", ctypes.c_int), ("flags", ctypes.c_int),
    ]

    @classmethod
    def from_params(cls, p) -> "CoParams":
        c = cls()
        c.dt, c.lam, c.myu, c.stiff_bend = p.dt, p.lam, p.myu, p.stiff_bend
        c.gravity[:] = list(p.gravity)
        c.mass_point, c.stiff_contact, c.contact_clearance = p.mass_point, p.stiff_contact, p.contact_clearance
        c.obs_center[:] = list(p.obs_center)
        c.obs_radius, c.tol = p.obs_radius, p.tol
        c.obstacle_kind, c.solver_kind, c.maxit = p.obstacle_kind, p.solver_kind, p.maxit
        return c


class CoStats(ctypes.Structure):
    _fields_ = [
        ("solver_iterations", ctypes.c_int), ("n_prx", ctypes.c_int), ("n_ccd_passes", ctypes.c_int),
        ("n_ccd", ctypes.c_int * 5), ("n_riz_passes", ctypes.c_int), ("n_riz_last", ctypes.c_int),
        ("n_riz_total", ctypes.c_int), ("riz_nodes", ctypes.c_int), ("impulse_applied", ctypes.c_int),
        ("ilu_singular", ctypes.c_int), ("solver_conv", ctypes.c_double),
    ]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["n_ccd"] = list(self.n_ccd)
        return d


def build(which: str = "port") -> str:
    """Build one oracle library with make; returns its path."""
    target = {"port": "port", "ref": "ref"}[which]
    args = ["make", "-s", "-C", HERE, target]
    if which == "ref":
        args.append("REF=" + REF_SRC)
    subprocess.run(args, check=True)
    return PORT_LIB if which == "port" else REF_LIB


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_V = ctypes.c_void_p


def _dp(a):
    return a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I)


class OracleLib:
    """One loaded oracle library (``port`` or ``ref``)."""

    def __init__(self, which: str = "port"):
        path = PORT_LIB if which == "port" else REF_LIB
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library {path} not built (oracle.build('{which}'))")
        self.which = which
        self.lib = ctypes.CDLL(path)
        pre = "co_" if which == "port" else "ref_"
        self.pre = pre
        L = self.lib

        def f(name, res, *args):
            fn = getattr(L, pre + name)
            fn.restype = res
            fn.argtypes = list(args)
            return fn

        P = ctypes.POINTER(CoParams)
        S = ctypes.POINTER(CoStats)
        self.create = f("create", _V, ctypes.c_int, _D, _I, ctypes.c_int, _I, ctypes.c_int, _I, P)
        self.destroy = f("destroy", None, _V)
        self.set_params = f("set_params", None, _V, P)
        self.num_blocks = f("num_blocks", ctypes.c_int, _V)
        self.pattern = f("pattern", None, _V, _I, _I)
        self.num_nodes = f("num_nodes", ctypes.c_int, _V)
        self.bvh_nodes = f("bvh_nodes", None, _V, _I)
        self.num_edges = f("num_edges", ctypes.c_int, _V)
        self.edges = f("edges", None, _V, _I, _I)
        self.wdwddw_cst = f("wdwddw_cst", None, _D, _D, ctypes.c_double, ctypes.c_double, _D, _D, _D)
        self.wdwddw_bend = f("wdwddw_bend", None, _D, _D, ctypes.c_double, _D, _D, _D)
        self.wdwddw_contact = f("wdwddw_contact", None, _D, P, _D, _D, _D)
        self.assemble = f("assemble", None, _V, _D, _D, _D, _D, _D)
        self.ilu = f("ilu", ctypes.c_int, _V, _D, _D)
        self.pcg = f("pcg", None, _V, _D, ctypes.c_double, ctypes.c_int, _D, _D, _I)
        self.cg = f("cg", None, _V, _D, ctypes.c_double, ctypes.c_int, _D, _D, _I)
        self.implicit = f("implicit", None, _V, _D, _D, S)
        self.refit_prx = f("refit_prx", None, _V, _D, ctypes.c_double, _D)
        self.refit_ccd = f("refit_ccd", None, _V, _D, _D, ctypes.c_double, _D)
        self.contacts_prx = f("contacts_prx", ctypes.c_int, _V, _D, ctypes.c_double, _I, ctypes.c_int)
        self.contacts_ccd = f("contacts_ccd", ctypes.c_int, _V, _D, _D, ctypes.c_double, ctypes.c_double,
                              _I, ctypes.c_int)
        self.impulse_prx = f("impulse_prx", None, _V, _D, _D, _I, ctypes.c_int)
        self.impulse_ccd = f("impulse_ccd", None, _V, _D, _D, _I, ctypes.c_int)
        self.riz_reset = f("riz_reset", None, _V)
        self.riz_add = f("riz_add", None, _V, _I, ctypes.c_int)
        self.riz_zones = f("riz_zones", ctypes.c_int, _V, _I)
        self.riz_apply = f("riz_apply", None, _V, _D, _D, _D)
        self.resolve = f("resolve", None, _V, _D, _D, S)
        self.update_velocity = f("update_velocity", None, _V, _D, _D)
        self.vertex_normals = f("vertex_normals", None, _V, _D, _D)
        self.step = f("step", None, _V, _D, _D, S)
        self.last_residual = f("last_residual", None, _V, _D)
        self.ilu_solve = f("ilu_solve", None, _V, _D)
        self.matvec = f("matvec", None, _V, ctypes.c_double, _D, ctypes.c_double, _D)
        self.distance_fv = f("distance_fv", ctypes.c_double, _D, _D)
        self.distance_ee = f("distance_ee", ctypes.c_double, _D, _D)
        self.coplanar_time = f("coplanar_time", ctypes.c_double, _D, _D)
        self.fv_ccd_batch = f("fv_ccd_batch", None, ctypes.c_int, _D, _D, _I)
        self.ee_ccd_batch = f("ee_ccd_batch", None, ctypes.c_int, _D, _I)
        # contact log (restatement only: the reference keeps no per-pass record)
        self.has_log = hasattr(L, pre + "contact_log")
        if self.has_log:
            self.contact_log = f("contact_log", None, _V, ctypes.c_int)
            self.contact_log_read = f("contact_log_read", ctypes.c_int, _V, _I, _I,
                                      ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int)
            self.contact_digest = f("contact_digest", ctypes.c_ulonglong, _I, ctypes.c_int)


class OracleCloth:
    """A cloth simulated by an oracle library, with numpy in/out."""

    def __init__(self, lib: OracleLib, cloth):
        self.L = lib
        self.cloth = cloth
        self.n = cloth.np
        self._X0 = np.ascontiguousarray(cloth.X0, dtype=np.float64)
        self._bc = np.ascontiguousarray(cloth.bc, dtype=np.int32)
        self._tri = np.ascontiguousarray(cloth.tri, dtype=np.int32)
        self._quad = np.ascontiguousarray(cloth.quad, dtype=np.int32)
        self.prm = CoParams.from_params(cloth.params)
        self.h = lib.create(self.n, _dp(self._X0), _ip(self._bc), cloth.nt, _ip(self._tri),
                            cloth.nq, _ip(self._quad), ctypes.byref(self.prm))
        self.x = self._X0.copy()
        self.v = np.zeros_like(self._X0)

    def close(self):
        if self.h:
            self.L.destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        self.prm = CoParams.from_params(params)
        self.L.set_params(self.h, ctypes.byref(self.prm))

    # topology
    def pattern(self):
        nb = self.L.num_blocks(self.h)
        rp = np.zeros(self.n + 1, np.int32)
        ci = np.zeros(nb, np.int32)
        self.L.pattern(self.h, _ip(rp), _ip(ci))
        return rp, ci

    def bvh_nodes(self):
        nn = self.L.num_nodes(self.h)
        out = np.zeros(3 * nn, np.int32)
        self.L.bvh_nodes(self.h, _ip(out))
        return out.reshape(nn, 3)

    def edges(self):
        ne = self.L.num_edges(self.h)
        idx = np.zeros(self.n + 1, np.int32)
        arr = np.zeros(ne, np.int32)
        self.L.edges(self.h, _ip(idx), _ip(arr))
        return idx, arr

    # implicit-step pieces
    def assemble(self, x, v):
        nb = self.L.num_blocks(self.h)
        vd = np.zeros(9 * self.n)
        vc = np.zeros(9 * nb)
        b = np.zeros(3 * self.n)
        self.L.assemble(self.h, _dp(np.ascontiguousarray(x)), _dp(np.ascontiguousarray(v)),
                        _dp(vd), _dp(vc), _dp(b))
        return vd, vc, b

    def ilu(self):
        nb = self.L.num_blocks(self.h)
        fd = np.zeros(9 * self.n)
        fc = np.zeros(9 * nb)
        ns = self.L.ilu(self.h, _dp(fd), _dp(fc))
        return fd, fc, ns

    def pcg(self, b, tol, maxit):
        x = np.zeros(3 * self.n)
        conv = ctypes.c_double()
        it = ctypes.c_int()
        self.L.pcg(self.h, _dp(np.ascontiguousarray(b)), tol, maxit, _dp(x), ctypes.byref(conv),
                   ctypes.byref(it))
        return x, conv.value, it.value

    def cg(self, b, tol, maxit):
        x = np.zeros(3 * self.n)
        conv = ctypes.c_double()
        it = ctypes.c_int()
        self.L.cg(self.h, _dp(np.ascontiguousarray(b)), tol, maxit, _dp(x), ctypes.byref(conv),
                  ctypes.byref(it))
        return x, conv.value, it.value

    def last_residual(self):
        """r_vec left by the last cg / pcg."""
        r = np.zeros(3 * self.n)
        self.L.last_residual(self.h, _dp(r))
        return r

    def ilu_solve(self, vec):
        """CPreconditionerILU::Solve with the last ilu() factor."""
        z = np.array(vec, dtype=np.float64)
        self.L.ilu_solve(self.h, _dp(z))
        return z

    def matvec(self, alpha, x, beta, y):
        """MatVec(alpha, x, beta, y) on the last assembled matrix."""
        y = np.array(y, dtype=np.float64)
        self.L.matvec(self.h, alpha, _dp(np.ascontiguousarray(x, dtype=np.float64)), beta, _dp(y))
        return y

    def implicit(self, x, v):
        x = np.array(x, dtype=np.float64)
        v = np.array(v, dtype=np.float64)
        st = CoStats()
        self.L.implicit(self.h, _dp(x), _dp(v), ctypes.byref(st))
        return x, v, st.as_dict()

    # collision pieces
    def refit_prx(self, x, delta):
        out = np.zeros(7 * self.L.num_nodes(self.h))
        self.L.refit_prx(self.h, _dp(np.ascontiguousarray(x)), delta, _dp(out))
        return out.reshape(-1, 7)

    def refit_ccd(self, x, v, dt):
        out = np.zeros(7 * self.L.num_nodes(self.h))
        self.L.refit_ccd(self.h, _dp(np.ascontiguousarray(x)), _dp(np.ascontiguousarray(v)), dt, _dp(out))
        return out.reshape(-1, 7)

    def contacts_prx(self, x, delta, cap=1 << 20):
        out = np.zeros(5 * cap, np.int32)
        n = self.L.contacts_prx(self.h, _dp(np.ascontiguousarray(x)), delta, _ip(out), cap)
        assert n <= cap
        return out[: 5 * n].reshape(n, 5)

    def contacts_ccd(self, x, v, dt, delta, cap=1 << 20):
        out = np.zeros(5 * cap, np.int32)
        n = self.L.contacts_ccd(self.h, _dp(np.ascontiguousarray(x)), _dp(np.ascontiguousarray(v)), dt,
                                delta, _ip(out), cap)
        assert n <= cap
        return out[: 5 * n].reshape(n, 5)

    def impulse_prx(self, x, v, ce):
        v = np.array(v, dtype=np.float64)
        ce = np.ascontiguousarray(ce, dtype=np.int32)
        self.L.impulse_prx(self.h, _dp(np.ascontiguousarray(x)), _dp(v), _ip(ce), ce.shape[0])
        return v

    def impulse_ccd(self, x, v, ce):
        v = np.array(v, dtype=np.float64)
        ce = np.ascontiguousarray(ce, dtype=np.int32)
        self.L.impulse_ccd(self.h, _dp(np.ascontiguousarray(x)), _dp(v), _ip(ce), ce.shape[0])
        return v

    def riz_reset(self):
        self.L.riz_reset(self.h)

    def riz_add(self, ce):
        ce = np.ascontiguousarray(ce, dtype=np.int32)
        self.L.riz_add(self.h, _ip(ce), ce.shape[0])

    def riz_zones(self):
        z = np.zeros(self.n, np.int32)
        nz = self.L.riz_zones(self.h, _ip(z))
        return z, nz

    def riz_apply(self, x, v, v0):
        v = np.array(v, dtype=np.float64)
        self.L.riz_apply(self.h, _dp(np.ascontiguousarray(x)), _dp(v), _dp(np.ascontiguousarray(v0)))
        return v

    def resolve(self, x1, v):
        v = np.array(v, dtype=np.float64)
        st = CoStats()
        self.L.resolve(self.h, _dp(np.ascontiguousarray(x1)), _dp(v), ctypes.byref(st))
        return v, st.as_dict()

    def update_velocity(self, x, v):
        v = np.array(v, dtype=np.float64)
        self.L.update_velocity(self.h, _dp(np.ascontiguousarray(x)), _dp(v))
        return v

    def vertex_normals(self, x):
        """MakeNormal (self_contact_sparse/main.cpp:183-211) at positions x."""
        out = np.zeros(3 * self.cloth.np)
        self.L.vertex_normals(self.h, _dp(np.ascontiguousarray(x, dtype=np.float64)), _dp(out))
        return out

    def log_contacts(self, enable: bool = True):
        """Record, per detection of the following resolve / step, (kind,
        count, digest of the ordered contact list)."""
        self.L.contact_log(self.h, int(enable))

    def contact_log(self):
        """The detections of the last resolve: a list of (ccd, count, digest)."""
        cap = 256
        while True:
            k = np.zeros(cap, np.int32)
            c = np.zeros(cap, np.int32)
            d = np.zeros(cap, np.uint64)
            n = self.L.contact_log_read(self.h, _ip(k), _ip(c),
                                        d.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong)), cap)
            if n <= cap:
                return [(int(k[i]), int(c[i]), int(d[i])) for i in range(n)]
            cap = n

    def step(self, nsteps: int = 1):
        stats = []
        for _ in range(nsteps):
            st = CoStats()
            self.L.step(self.h, _dp(self.x), _dp(self.v), ctypes.byref(st))
            stats.append(st.as_dict())
        return stats


def wdwddw_cst(lib: OracleLib, C, c, lam, myu):
    W = ctypes.c_double()
    dW = np.zeros(9)
    ddW = np.zeros(81)
    lib.wdwddw_cst(_dp(np.ascontiguousarray(C, np.float64)), _dp(np.ascontiguousarray(c, np.float64)),
                   lam, myu, ctypes.byref(W), _dp(dW), _dp(ddW))
    return W.value, dW, ddW


def wdwddw_bend(lib: OracleLib, C, c, stiff):
    W = ctypes.c_double()
    dW = np.zeros(12)
    ddW = np.zeros(144)
    lib.wdwddw_bend(_dp(np.ascontiguousarray(C, np.float64)), _dp(np.ascontiguousarray(c, np.float64)),
                    stiff, ctypes.byref(W), _dp(dW), _dp(ddW))
    return W.value, dW, ddW


def wdwddw_contact(lib: OracleLib, c, params):
    W = ctypes.c_double()
    dW = np.zeros(3)
    ddW = np.zeros(9)
    prm = CoParams.from_params(params)
    lib.wdwddw_contact(_dp(np.ascontiguousarray(c, np.float64)), ctypes.byref(prm), ctypes.byref(W),
                       _dp(dW), _dp(ddW))
    return W.value, dW, ddW


def distance_fv(lib: OracleLib, pts):
    """DistanceFaceVertex on 12 doubles (face p0 p1 p2, vertex p3): (dist, w0, w1)."""
    w = np.zeros(2)
    d = lib.distance_fv(_dp(np.ascontiguousarray(pts, dtype=np.float64)), _dp(w))
    return d, w[0], w[1]


def distance_ee(lib: OracleLib, pts):
    """DistanceEdgeEdge on 12 doubles (p0 p1 q0 q1): (dist, ratio_p, ratio_q)."""
    r = np.zeros(2)
    d = lib.distance_ee(_dp(np.ascontiguousarray(pts, dtype=np.float64)), _dp(r))
    return d, r[0], r[1]


def coplanar_time(lib: OracleLib, s, e):
    """FindCoplanerInterp on start / end points (12 doubles each)."""
    return lib.coplanar_time(_dp(np.ascontiguousarray(s, dtype=np.float64)),
                             _dp(np.ascontiguousarray(e, dtype=np.float64)))


def fv_ccd(lib: OracleLib, pts, box=None) -> np.ndarray:
    """IsContact_FV_CCD on configurations (n, 24): start face p0 p1 p2, vertex
    p3, then their end points; box (6: lo, hi) for the face's node, by default
    one that holds everything.  0 / 1 per configuration."""
    p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 24)
    b = np.ascontiguousarray(box if box is not None else [-1e30] * 3 + [1e30] * 3, dtype=np.float64)
    out = np.zeros(len(p), dtype=np.int32)
    lib.fv_ccd_batch(len(p), _dp(p), _dp(b), out.ctypes.data_as(_I))
    return out


def ee_ccd(lib: OracleLib, pts) -> np.ndarray:
    """IsContact_EE_CCD on configurations (n, 24): start edges p0 p1, q0 q1,
    then their end points.  0 / 1 per configuration."""
    p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 24)
    out = np.zeros(len(p), dtype=np.int32)
    lib.ee_ccd_batch(len(p), _dp(p), out.ctypes.data_as(_I))
    return out
