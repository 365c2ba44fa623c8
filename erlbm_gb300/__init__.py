"""erlbm_gb300 -- GB300 (sm_103a) engine for the E-RLBM collide-stream path of SimBoltz / ERLBM.

The compute lives in liberlbm_gb300.so (hand-written CUDA behind the C ABI of
include/erlbm_gb300.h).  This package is a thin host-side mirror of that ABI with the reference's
vocabulary: a ``Lattice`` is what define_rede + aloca_populacoes build (src/erlbm_common.h:123-148),
``Lattice.step`` is one pass of a driver's collide+propagate node loop plus the pointer swap,
``Lattice.run`` is roda_ponto, and ``map_run`` is a whole stability-map sweep.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import (FP32_SHIFTED, FP64, MAP_OBSTACLE, MAP_TAYLOR_GREEN, OP_BGK, OP_EXTREG, OP_MRT, OP_REG,
                   STAGE_POST_COLLISION, STAGE_POST_STREAM, ErlbmError, check, lib)

__all__ = ["Lattice", "ErlbmError", "lib", "OP_BGK", "OP_MRT", "OP_REG", "OP_EXTREG", "FP64", "FP32_SHIFTED",
           "STAGE_POST_STREAM", "STAGE_POST_COLLISION", "MAP_TAYLOR_GREEN", "MAP_OBSTACLE", "init_taylor_green",
           "init_double_shear", "equilibrium", "obstacle_geometry", "taylor_green_error", "tg_map_params",
           "obstacle_map_params", "operator_from_name"]

_OPS = {"bgk": OP_BGK, "mrt": OP_MRT, "reg": OP_REG, "erlbm": OP_EXTREG}


def operator_from_name(name: str) -> int:
    """le_colisao (src/erlbm_common.h:44-54), raising instead of exit(1) on an unknown name."""
    try:
        return _OPS[name]
    except KeyError:
        raise ValueError(f"unknown collision operator {name!r} (use bgk, mrt, reg or erlbm)") from None


def _dptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Lattice:
    """One lattice on the GPU.  Populations cross the boundary as AoS doubles in fluid-index order."""

    def __init__(self, q: int, nx: int, ny: int, nz: int = 1, solid=None, tau: float = 0.6, tau_nh: float = 0.65,
                 op: int = OP_EXTREG, precision: int = FP64):
        L = lib()
        self._solid = None
        sp = None
        if solid is not None:
            self._solid = np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1)
            if self._solid.size != nx * ny * nz:
                raise ValueError("solid mask must have nx * ny * nz entries")
            sp = self._solid.ctypes.data
        d = _lib.Desc(q, nx, ny, nz, sp, tau, tau_nh, op, precision)
        h = C.c_void_p()
        check(L.erlbm_create(C.byref(d), C.byref(h)), "erlbm_create")
        self._h = h
        self.q, self.nx, self.ny, self.nz, self.precision = q, nx, ny, nz, precision
        n = C.c_int64()
        check(L.erlbm_fluid_count(h, C.byref(n)), "erlbm_fluid_count")
        self.n_fluid = n.value

    def close(self):
        if getattr(self, "_h", None):
            lib().erlbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_params(self, tau: float, tau_nh: float, op: int):
        check(lib().erlbm_set_params(self._h, tau, tau_nh, op), "erlbm_set_params")

    def set_populations(self, f) -> None:
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        check(lib().erlbm_set_populations(self._h, _dptr(f), f.size), "erlbm_set_populations")

    def get_populations(self, stage: int = STAGE_POST_STREAM, out=None) -> np.ndarray:
        if out is None:
            out = np.empty(self.n_fluid * self.q, dtype=np.float64)
        check(lib().erlbm_get_populations(self._h, _dptr(out), out.size, stage), "erlbm_get_populations")
        return out

    def step(self, n: int = 1, bc: dict | None = None) -> None:
        b = _bc(bc)
        check(lib().erlbm_step(self._h, int(n), C.byref(b) if b is not None else None), "erlbm_step")

    def sync(self) -> None:
        check(lib().erlbm_sync(self._h), "erlbm_sync")

    def kinetic_energy(self, stage: int = STAGE_POST_STREAM) -> float:
        e = C.c_double()
        check(lib().erlbm_kinetic_energy(self._h, stage, C.byref(e)), "erlbm_kinetic_energy")
        return e.value

    def max_abs_density(self, stage: int = STAGE_POST_STREAM):
        m, nf = C.c_double(), C.c_int()
        check(lib().erlbm_max_abs_density(self._h, stage, C.byref(m), C.byref(nf)), "erlbm_max_abs_density")
        return m.value, bool(nf.value)

    def macroscopic(self, stage: int = STAGE_POST_STREAM):
        rho = np.empty(self.n_fluid)
        u = np.empty((self.n_fluid, 3))
        check(lib().erlbm_macroscopic(self._h, stage, _dptr(rho), _dptr(u)), "erlbm_macroscopic")
        return rho, u

    def run(self, n_steps: int, bc: dict | None = None, energy_every: int = 0, energy_factor: float = 2.0,
            density_check: bool = False, density_limit: float = 10.0) -> dict:
        b = _bc(bc)
        c = _lib.Checks(int(energy_every), float(energy_factor), int(bool(density_check)), float(density_limit))
        r = _lib.RunResult()
        check(lib().erlbm_run(self._h, int(n_steps), C.byref(b) if b is not None else None, C.byref(c), C.byref(r)),
              "erlbm_run")
        return dict(label=r.label, decided_step=r.decided_step, steps_done=r.steps_done, margin=r.margin)


def _bc(bc: dict | None):
    if bc is None:
        return None
    return _lib.BC(int(bc.get("inlet_x", -1)), float(bc.get("u_in", 0.0)), int(bc.get("outlet_x", -1)),
                   float(bc.get("rho_out", 1.0)))


# ---- program inputs (host functions of the library) --------------------------------------------

def _fn(name, res, args):
    f = getattr(lib(), name)
    f.restype = res
    f.argtypes = args
    return f


def init_taylor_green(q: int, L: int, u0: float, tau: float, poisson=True, neq=True, variant=0, nz=1) -> np.ndarray:
    out = np.empty(L * L * nz * q)
    f = _fn("erlbm_init_taylor_green", C.c_int, [C.c_int] * 3 + [C.c_double] * 2 + [C.c_int] * 3 + [C.c_void_p])
    check(f(q, L, nz, u0, tau, int(poisson), int(neq), int(variant), _dptr(out)), "erlbm_init_taylor_green")
    return out


def init_double_shear(L: int, rho: float = 1.0) -> np.ndarray:
    out = np.empty(L * L * 9)
    f = _fn("erlbm_init_double_shear", C.c_int, [C.c_int, C.c_double, C.c_void_p])
    check(f(L, rho, _dptr(out)), "erlbm_init_double_shear")
    return out


def equilibrium(q: int, ux: float, uy: float, uz: float, rho: float) -> np.ndarray:
    out = np.empty(q)
    f = _fn("erlbm_equilibrium", C.c_int, [C.c_int] + [C.c_double] * 4 + [C.c_void_p])
    check(f(q, ux, uy, uz, rho, _dptr(out)), "erlbm_equilibrium")
    return out


def obstacle_geometry(sx: int = 1, sy: int = 1):
    f = _fn("erlbm_obstacle_geometry", C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p])
    nx, ny = C.c_int(), C.c_int()
    check(f(sx, sy, C.byref(nx), C.byref(ny), None), "erlbm_obstacle_geometry")
    solid = np.zeros(nx.value * ny.value, dtype=np.uint8)
    check(f(sx, sy, C.byref(nx), C.byref(ny), _dptr(solid)), "erlbm_obstacle_geometry")
    return nx.value, ny.value, solid


def taylor_green_error(q: int, L: int, f, u0: float, visc: float, step: int, variant: int = 0):
    f = np.ascontiguousarray(f, dtype=np.float64)
    out = np.empty(3)
    fn = _fn("erlbm_taylor_green_error", C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_int,
                                                   C.c_int, C.c_void_p])
    check(fn(q, L, _dptr(f), u0, visc, step, variant, _dptr(out)), "erlbm_taylor_green_error")
    return out


def tg_map_params(i: int, j: int, n_ma: int = 400, n_nu: int = 400, op: int = OP_EXTREG, tau_nh: float = 0.65):
    fn = _fn("erlbm_tg_map_params", C.c_int, [C.c_int] * 5 + [C.c_double] + [C.POINTER(C.c_double)] * 3)
    a, b, c = C.c_double(), C.c_double(), C.c_double()
    check(fn(i, j, n_ma, n_nu, op, tau_nh, C.byref(a), C.byref(b), C.byref(c)), "erlbm_tg_map_params")
    return a.value, b.value, c.value


def obstacle_map_params(i: int, j: int, n_tau: int = 400, n_nu: int = 400, ma: float = 0.1):
    fn = _fn("erlbm_obstacle_map_params", C.c_int, [C.c_int] * 4 + [C.c_double] + [C.POINTER(C.c_double)] * 3)
    a, b, c = C.c_double(), C.c_double(), C.c_double()
    check(fn(i, j, n_tau, n_nu, ma, C.byref(a), C.byref(b), C.byref(c)), "erlbm_obstacle_map_params")
    return a.value, b.value, c.value
