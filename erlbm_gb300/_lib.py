"""ctypes binding of liberlbm_gb300.so (declared in include/erlbm_gb300.h).

The library is the only compute path: if it cannot be built or loaded, ``lib()`` raises, and no
Python code falls back to another implementation.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liberlbm_gb300.so")

OK, E_INVAL, E_OOM, E_CUDA, E_TIMEOUT, E_NONFINITE, E_UNSUPPORTED, E_STATE = 0, -1, -2, -3, -4, -5, -6, -7
OP_BGK, OP_MRT, OP_REG, OP_EXTREG = 1, 2, 3, 4
FP64, FP32_SHIFTED, FP32_PAIR = 0, 1, 2
STAGE_POST_STREAM, STAGE_POST_COLLISION = 0, 1
MAP_TAYLOR_GREEN, MAP_OBSTACLE = 1, 2
INIT_REST, INIT_TG_MAP, INIT_AOS = 0, 1, 2
REQ_TG2D, REQ_TG_MAP_POINT, REQ_OBSTACLE, REQ_TG3D = 1, 2, 3, 4
FIELD_VELOCITY, FIELD_VORTICITY, FIELD_DENSITY = 1, 2, 3
VTK_ASCII, VTK_BINARY_FLOAT, VTK_BINARY_DOUBLE = 0, 1, 2


class ErlbmError(RuntimeError):
    def __init__(self, code: int, what: str, detail: str):
        super().__init__(f"{what}: {detail} (status {code})")
        self.code = code


class Desc(C.Structure):
    _fields_ = [("q", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("solid", C.c_void_p),
                ("tau", C.c_double), ("tau_nh", C.c_double), ("op", C.c_int), ("precision", C.c_int)]


INLET_ZOUHE, INLET_PARABOLIC = 0, 1
OUTLET_DENSITY, OUTLET_OPEN, OUTLET_CONVECTIVE = 0, 1, 2


class BC(C.Structure):
    _fields_ = [("inlet_x", C.c_int), ("u_in", C.c_double), ("outlet_x", C.c_int), ("rho_out", C.c_double),
                ("inlet_kind", C.c_int), ("parabolic_L", C.c_int), ("outlet_kind", C.c_int), ("open_y_on", C.c_int),
                ("open_y", C.c_int)]


class Checks(C.Structure):
    _fields_ = [("energy_every", C.c_int), ("energy_factor", C.c_double), ("density_check", C.c_int),
                ("density_limit", C.c_double)]


class RunResult(C.Structure):
    _fields_ = [("label", C.c_int), ("decided_step", C.c_int), ("steps_done", C.c_int), ("margin", C.c_double)]


class MapDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("precision", C.c_int), ("op", C.c_int), ("tau_nh", C.c_double), ("L", C.c_int),
                ("ma", C.c_double), ("n_i", C.c_int), ("n_j", C.c_int), ("n_points", C.c_int),
                ("pi", C.c_void_p), ("pj", C.c_void_p), ("max_steps", C.c_int), ("slots", C.c_int)]


class RefineDesc(C.Structure):
    _fields_ = [("radius", C.c_int), ("late_fraction", C.c_double), ("probe_stride", C.c_int),
                ("max_passes", C.c_int)]


class BatchDesc(C.Structure):
    _fields_ = [("q", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("solid", C.c_void_p), ("inlet_x", C.c_int),
                ("outlet_x", C.c_int), ("rho0", C.c_double), ("energy_every", C.c_int),
                ("energy_factor", C.c_double), ("density_check", C.c_int), ("density_limit", C.c_double),
                ("init", C.c_int), ("precision", C.c_int), ("slots", C.c_int)]


class RunSpec(C.Structure):
    _fields_ = [("op", C.c_int), ("tau", C.c_double), ("tau_nh", C.c_double), ("u0", C.c_double),
                ("n_steps", C.c_int), ("aos_offset", C.c_int64)]


class BatchResult(C.Structure):
    _fields_ = [("label", C.c_int), ("decided_step", C.c_int), ("steps_done", C.c_int), ("status", C.c_int),
                ("margin", C.c_double), ("energy", C.c_double)]


class ServerDesc(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_longlong), ("slot_ctas", C.c_int), ("max_streams", C.c_int),
                ("queue_capacity", C.c_int), ("team_ctas", C.c_int), ("team_max_nodes", C.c_int),
                ("team_wait_us", C.c_int)]


class Request(C.Structure):
    _fields_ = [("kind", C.c_int), ("precision", C.c_int), ("op", C.c_int), ("L", C.c_int), ("sx", C.c_int),
                ("sy", C.c_int), ("tau", C.c_double), ("tau_nh", C.c_double), ("u0", C.c_double),
                ("n_steps", C.c_int)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("label", C.c_int), ("steps_done", C.c_int), ("decided_step", C.c_int),
                ("energy", C.c_double), ("margin", C.c_double), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("lane", C.c_int)]


_lock = threading.Lock()
_lib = None

_SIGS = {
    "erlbm_version": (C.c_int, []),
    "erlbm_strerror": (C.c_char_p, [C.c_int]),
    "erlbm_last_error": (C.c_char_p, []),
    "erlbm_create": (C.c_int, [C.POINTER(Desc), C.POINTER(C.c_void_p)]),
    "erlbm_destroy": (C.c_int, [C.c_void_p]),
    "erlbm_fluid_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "erlbm_set_params": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int]),
    "erlbm_set_populations": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "erlbm_get_populations": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]),
    "erlbm_step": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(BC)]),
    "erlbm_kinetic_energy": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "erlbm_max_abs_density": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "erlbm_macroscopic": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "erlbm_field": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_size_t]),
    "erlbm_read_geo": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                 C.POINTER(C.c_int), C.c_void_p, C.c_size_t]),
    "erlbm_write_vtk": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_char_p]),
    "erlbm_velocity_error": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]),
    "erlbm_run": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(BC), C.POINTER(Checks), C.POINTER(RunResult)]),
    "erlbm_sync": (C.c_int, [C.c_void_p]),
    "erlbm_fp64_rate": (C.c_int, [C.POINTER(C.c_double)]),
    "erlbm_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "erlbm_set_launch": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "erlbm_batch_run": (C.c_int, [C.POINTER(BatchDesc), C.c_int, C.POINTER(RunSpec), C.c_void_p, C.c_size_t,
                                  C.POINTER(BatchResult)]),
    "erlbm_map_run": (C.c_int, [C.POINTER(MapDesc), C.c_void_p, C.c_void_p, C.c_void_p]),
    "erlbm_map_run_refined": (C.c_int, [C.POINTER(MapDesc), C.POINTER(RefineDesc), C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]),
    "erlbm_server_start": (C.c_int, [C.POINTER(ServerDesc), C.POINTER(C.c_void_p)]),
    "erlbm_server_submit": (C.c_int, [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_int64)]),
    "erlbm_server_poll": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(Result)]),
    "erlbm_server_wait": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(Result), C.c_double]),
    "erlbm_server_clock": (C.c_double, [C.c_void_p]),
    "erlbm_server_stop": (C.c_int, [C.c_void_p]),
}


def lib():
    """Build (when sources are newer) and load liberlbm_gb300.so; raises if that is impossible."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        from . import build as _build
        path = _build.build()
        L = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            if hasattr(L, name):
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
        _lib = L
        return L


def check(code: int, what: str) -> None:
    if code != OK:
        detail = lib().erlbm_last_error().decode(errors="replace") or lib().erlbm_strerror(code).decode()
        raise ErlbmError(code, what, detail)
