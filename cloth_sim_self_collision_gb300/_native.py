"""ctypes binding of the C ABI in include/clothgpu.h (lib/libclothgpu.so).

There is no CPU fallback: loading fails loudly when the library is missing or
no GPU is present.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB

CS_OK = 0
CS_ERR_ARG = 1
CS_ERR_CUDA = 2
CS_ERR_NO_DEVICE = 3
CS_ERR_OOM = 4
CS_ERR_CAPACITY = 5
CS_ERR_TIMEOUT = 6
CS_ERR_DIVERGED = 7

CS_FLAG_EXACT_DOTS = 1

CS_PREC_FP64 = 0
CS_PREC_MIXED = 1

# every entry point declared in include/clothgpu.h
EXPORTS = [
    "cs_create", "cs_destroy", "cs_last_error", "cs_set_precision", "cs_synchronize", "cs_add_cloth",
    "cs_remove_cloth", "cs_num_cloths", "cs_set_params", "cs_set_state", "cs_get_state", "cs_get_stats",
    "cs_step", "cs_implicit_step", "cs_resolve_contacts", "cs_update_velocity", "cs_assemble", "cs_pattern",
    "cs_ilu_factor", "cs_solve_pcg", "cs_solve_cg", "cs_spmv", "cs_bvh_nodes", "cs_refit_prx", "cs_refit_ccd",
    "cs_contacts_prx", "cs_contacts_ccd", "cs_impulse_prx", "cs_impulse_ccd", "cs_riz_reset", "cs_riz_add",
    "cs_riz_zones", "cs_riz_apply", "cs_element_cst", "cs_element_bend", "cs_element_contact",
    "cs_launch_count", "cs_build_bvh", "cs_build_pattern", "cs_set_states", "cs_get_states", "cs_num_vertices",
    "cs_profile", "cs_profile_read", "cs_stream", "cs_profile_bytes", "cs_get_boxes", "cs_solve_cg_noalloc",
    "cs_server_create", "cs_server_submit", "cs_server_wait", "cs_server_release", "cs_server_drain",
    "cs_server_get_stats", "cs_server_last_error", "cs_server_destroy", "cs_scene_device_bytes",
    "cs_vertex_normals", "cs_contact_log", "cs_contact_log_read", "cs_matvec", "cs_set_matrix", "cs_ilu_solve",
    "cs_distance_fv", "cs_distance_ee", "cs_coplanar_time", "cs_last_residual", "cs_set_frame_mode",
    "cs_frame_counts", "cs_frame_overflows", "cs_autotune",
]


class CsTuneResult(ctypes.Structure):
    _fields_ = [("mx_blocks_per_sm", ctypes.c_int), ("mx_tail_slices", ctypes.c_int),
                ("graph_grid_per_sm", ctypes.c_int), ("narrow_regs", ctypes.c_int),
                ("bar_sleep_ns", ctypes.c_int), ("impulse_cluster", ctypes.c_int), ("frame_ms", ctypes.c_double),
                ("candidates", ctypes.c_int),
                ("cached", ctypes.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class CsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"clothgpu error {code}: {msg}")
        self.code = code


class CsParams(ctypes.Structure):
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
    def from_params(cls, p) -> "CsParams":
        c = cls()
        c.dt, c.lam, c.myu, c.stiff_bend = p.dt, p.lam, p.myu, p.stiff_bend
        c.gravity[:] = list(p.gravity)
        c.mass_point, c.stiff_contact, c.contact_clearance = p.mass_point, p.stiff_contact, p.contact_clearance
        c.obs_center[:] = list(p.obs_center)
        c.obs_radius, c.tol = p.obs_radius, p.tol
        c.obstacle_kind, c.solver_kind, c.maxit = p.obstacle_kind, p.solver_kind, p.maxit
        c.flags = getattr(p, "flags", 0)
        return c


class CsStats(ctypes.Structure):
    _fields_ = [
        ("solver_iterations", ctypes.c_int), ("n_prx", ctypes.c_int), ("n_ccd_passes", ctypes.c_int),
        ("n_ccd", ctypes.c_int * 5), ("n_riz_passes", ctypes.c_int), ("n_riz_last", ctypes.c_int),
        ("n_riz_total", ctypes.c_int), ("riz_nodes", ctypes.c_int), ("impulse_applied", ctypes.c_int),
        ("ilu_singular", ctypes.c_int), ("solver_conv", ctypes.c_double), ("diverged", ctypes.c_int),
    ]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["n_ccd"] = list(self.n_ccd)
        return d


class CsServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("precision", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_double),
                ("max_cloths", ctypes.c_int)]


class CsRequestInfo(ctypes.Structure):
    _fields_ = [("np", ctypes.c_int), ("nsteps", ctypes.c_int), ("steps_done", ctypes.c_int),
                ("status", ctypes.c_int), ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double),
                ("t_first_frame", ctypes.c_double), ("t_done", ctypes.c_double),
                ("step_ms_p50", ctypes.c_double), ("step_ms_p99", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class CsServerStats(ctypes.Structure):
    _fields_ = [("frames", ctypes.c_longlong), ("vertex_steps", ctypes.c_longlong),
                ("submitted", ctypes.c_int), ("finished", ctypes.c_int), ("queued", ctypes.c_int),
                ("resident", ctypes.c_int), ("rebuilds", ctypes.c_int), ("diverged", ctypes.c_int),
                ("elapsed_s", ctypes.c_double), ("busy_s", ctypes.c_double),
                ("step_ms_p50", ctypes.c_double), ("step_ms_p99", ctypes.c_double),
                ("step_ms_max", ctypes.c_double), ("admit_ms_p50", ctypes.c_double),
                ("admit_ms_p99", ctypes.c_double), ("build_ms_total", ctypes.c_double),
                ("install_ms_total", ctypes.c_double), ("arena_bytes", ctypes.c_double),
                ("peak_bytes", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_V = ctypes.c_void_p
_lib = None


def load(path: str | None = None, build_if_missing: bool = False):
    """Loads the library (optionally building it first).  Raises when absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise FileNotFoundError(f"{path} not built: run cloth_sim_self_collision_gb300/build.py")
        _build.build()
    L = ctypes.CDLL(path)

    def f(name, res, *args):
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = list(args)

    P = ctypes.POINTER(CsParams)
    S = ctypes.POINTER(CsStats)
    i, d = ctypes.c_int, ctypes.c_double
    f("cs_create", i, i, i, ctypes.POINTER(_V))
    f("cs_destroy", None, _V)
    f("cs_last_error", ctypes.c_char_p, _V)
    f("cs_set_precision", i, _V, i)
    f("cs_synchronize", i, _V)
    f("cs_add_cloth", i, _V, i, _D, _I, i, _I, i, _I, P, _I)
    f("cs_remove_cloth", i, _V, i)
    f("cs_num_cloths", i, _V)
    f("cs_set_params", i, _V, i, P)
    f("cs_set_state", i, _V, i, _D, _D)
    f("cs_get_state", i, _V, i, _D, _D)
    f("cs_get_stats", i, _V, i, S)
    f("cs_step", i, _V, i)
    f("cs_implicit_step", i, _V, i, _D, _D, S)
    f("cs_resolve_contacts", i, _V, i, _D, _D, S)
    f("cs_update_velocity", i, _V, i, _D, _D)
    f("cs_assemble", i, _V, i, _D, _D, _D, _D, _D)
    f("cs_pattern", i, _V, i, _I, _I, _I)
    f("cs_ilu_factor", i, _V, i, _D, _D, _I)
    f("cs_solve_pcg", i, _V, i, _D, d, i, _D, _D, _I)
    f("cs_solve_cg", i, _V, i, _D, d, i, _D, _D, _I)
    f("cs_spmv", i, _V, i, _D, _D)
    f("cs_bvh_nodes", i, _V, i, _I, _I)
    f("cs_refit_prx", i, _V, i, _D, d, _D)
    f("cs_refit_ccd", i, _V, i, _D, _D, d, _D)
    f("cs_contacts_prx", i, _V, i, _D, d, _I, i, _I)
    f("cs_contacts_ccd", i, _V, i, _D, _D, d, d, _I, i, _I)
    f("cs_impulse_prx", i, _V, i, _D, _D, _I, i)
    f("cs_impulse_ccd", i, _V, i, _D, _D, _I, i)
    f("cs_riz_reset", i, _V, i)
    f("cs_riz_add", i, _V, i, _I, i)
    f("cs_riz_zones", i, _V, i, _I, _I)
    f("cs_riz_apply", i, _V, i, _D, _D, _D)
    f("cs_element_cst", i, _V, i, _D, _D, d, d, _D, _D, _D)
    f("cs_element_bend", i, _V, i, _D, _D, d, _D, _D, _D)
    f("cs_element_contact", i, _V, i, _D, P, _D, _D, _D)
    f("cs_launch_count", ctypes.c_longlong, _V)
    f("cs_build_bvh", i, i, _D, i, _I, _I, i, _I)
    f("cs_build_pattern", i, i, i, _I, _I, _I, i, _I)
    f("cs_set_states", i, _V, _D, _D)
    f("cs_get_states", i, _V, _D, _D)
    f("cs_num_vertices", ctypes.c_longlong, _V)
    f("cs_profile", i, _V, i)
    f("cs_stream", _V, _V)
    f("cs_get_boxes", i, _V, i, _D)
    f("cs_solve_cg_noalloc", i, _V, _V, _V, _V, _V, _V, i, d, i, _D, _I, _V)
    f("cs_profile_bytes", i, _V, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong))
    f("cs_profile_read", i, _V, ctypes.c_char_p, _D, ctypes.POINTER(ctypes.c_longlong))
    f("cs_server_create", i, ctypes.POINTER(CsServerConfig), ctypes.POINTER(_V))
    f("cs_server_submit", i, _V, i, _D, _I, i, _I, i, _I, _D, _D, P, i, _I)
    f("cs_server_wait", i, _V, i, d, _D, _D, ctypes.POINTER(CsRequestInfo))
    f("cs_server_release", i, _V, i)
    f("cs_server_drain", i, _V, d)
    f("cs_server_get_stats", i, _V, ctypes.POINTER(CsServerStats))
    f("cs_server_last_error", ctypes.c_char_p, _V)
    f("cs_server_destroy", None, _V)
    f("cs_scene_device_bytes", ctypes.c_size_t, i, _D, i, _I, i, _I, P)
    f("cs_vertex_normals", i, _V, i, _D, _D)
    f("cs_contact_log", i, _V, i)
    f("cs_set_frame_mode", i, _V, i)
    f("cs_autotune", i, _V, i, ctypes.POINTER(CsTuneResult))
    LL = ctypes.POINTER(ctypes.c_longlong)
    f("cs_frame_counts", i, _V, LL, LL, LL, LL)
    f("cs_frame_overflows", i, _V, LL)
    f("cs_matvec", i, _V, i, d, _D, d, _D)
    f("cs_last_residual", i, _V, i, _D)
    f("cs_set_matrix", i, _V, i, _D, _D)
    f("cs_ilu_solve", i, _V, i, _D)
    f("cs_distance_fv", i, _V, i, _D, _D, _D)
    f("cs_distance_ee", i, _V, i, _D, _D, _D)
    f("cs_coplanar_time", i, _V, i, _D, _D, _D)
    f("cs_contact_log_read", i, _V, i, _I, _I, ctypes.POINTER(ctypes.c_ulonglong), i, _I)
    _lib = L
    return L


def dp(a: np.ndarray):
    return a.ctypes.data_as(_D)


def ip(a: np.ndarray):
    return a.ctypes.data_as(_I)
