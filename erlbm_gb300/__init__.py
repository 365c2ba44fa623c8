"""erlbm_gb300 -- GB300 (sm_103a) engine for the E-RLBM collide-stream path of SimBoltz / ERLBM.

The compute lives in liberlbm_gb300.so (hand-written CUDA behind the C ABI of
include/erlbm_gb300.h).  This package is a thin host-side mirror of that ABI with the reference's
vocabulary: a ``Lattice`` is what define_rede + aloca_populacoes build (src/erlbm_common.h:123-148),
``Lattice.step`` is one pass of a driver's collide+propagate node loop plus the pointer swap,
``Lattice.run`` is roda_ponto, and ``map_run`` is a whole stability-map sweep.
"""
from __future__ import annotations

import ctypes as C
import os

# The request server keeps persistent kernels resident on their own streams.  Streams share the
# device's hardware work queues (8 unless this is set before the process creates its CUDA context),
# and a kernel queued behind a resident loop on a shared queue waits until that loop leaves.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np

from . import _lib
from ._lib import (FIELD_DENSITY, FIELD_VELOCITY, FIELD_VORTICITY, FP32_PAIR, FP32_SHIFTED, FP64, INIT_AOS, INIT_REST,
                   INIT_TG_MAP, INLET_PARABOLIC, INLET_ZOUHE, MAP_OBSTACLE, MAP_TAYLOR_GREEN, OP_BGK, OP_EXTREG,
                   OP_MRT, OP_REG, OUTLET_CONVECTIVE, OUTLET_DENSITY, OUTLET_OPEN, REQ_OBSTACLE,
                   REQ_TG2D, REQ_TG3D, REQ_TG_MAP_POINT, STAGE_POST_COLLISION, STAGE_POST_STREAM, VTK_ASCII,
                   VTK_BINARY_DOUBLE, VTK_BINARY_FLOAT, ErlbmError, check, lib)

__all__ = ["Lattice", "ErlbmError", "lib", "OP_BGK", "OP_MRT", "OP_REG", "OP_EXTREG", "FP64", "FP32_SHIFTED",
           "STAGE_POST_STREAM", "STAGE_POST_COLLISION", "MAP_TAYLOR_GREEN", "MAP_OBSTACLE", "init_taylor_green",
           "init_double_shear", "equilibrium", "obstacle_geometry", "taylor_green_error", "tg_map_params",
           "obstacle_map_params", "operator_from_name", "map_run", "map_run_refined", "batch_run", "INIT_REST",
           "INIT_TG_MAP", "INIT_AOS", "Server", "REQ_TG2D", "REQ_TG_MAP_POINT", "REQ_OBSTACLE", "REQ_TG3D",
           "FIELD_VELOCITY", "FIELD_VORTICITY", "FIELD_DENSITY", "VTK_ASCII", "VTK_BINARY_FLOAT",
           "VTK_BINARY_DOUBLE", "velocity_error", "INLET_ZOUHE", "INLET_PARABOLIC", "OUTLET_DENSITY", "OUTLET_OPEN",
           "OUTLET_CONVECTIVE", "read_geo"]

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

    def set_stream(self, stream_handle: int | None) -> None:
        """Queue the lattice's work on a caller's cudaStream_t (an int handle; None = own stream)."""
        check(lib().erlbm_set_stream(self._h, C.c_void_p(stream_handle) if stream_handle else None),
              "erlbm_set_stream")

    def set_launch(self, block_threads: int = 0, streaming_stores: bool = False, two_step: bool = False,
                   three_step: bool = False, wide_strips: bool = False) -> None:
        """Launch shape of the fused periodic D2Q9 FP32 kernel (see erlbm_gb300.autotune): two_step or
        three_step run two or three consecutive steps as one launch (nx % 128 == 0, ny even);
        wide_strips (with three_step) uses 64-column strips over column pairs; the same bits in every
        shape."""
        flags = ((1 if streaming_stores else 0) | (2 if two_step else 0) | (4 if three_step else 0) |
                 (8 if wide_strips else 0))
        check(lib().erlbm_set_launch(self._h, int(block_threads), flags), "erlbm_set_launch")

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

    def field(self, kind: int = FIELD_VELOCITY, stage: int = STAGE_POST_COLLISION) -> np.ndarray:
        """A field of the reference's writers at every box node (x fastest, solid nodes 0), computed on
        the device: velocity or vorticity as (n, 3), density as (n,)."""
        n = self.nx * self.ny * self.nz
        out = np.empty(n if kind == FIELD_DENSITY else (n, 3))
        check(lib().erlbm_field(self._h, stage, kind, _dptr(out), out.size), "erlbm_field")
        return out

    def write_vtk(self, path: str, kind: int = FIELD_VELOCITY, fmt: int = VTK_ASCII,
                  stage: int = STAGE_POST_COLLISION) -> None:
        """The field as a legacy VTK file, byte for byte what rec_velocity / rec_vorticity / rec_density
        (fmt VTK_ASCII) or their _bin variants (VTK_BINARY_FLOAT / _DOUBLE) write."""
        check(lib().erlbm_write_vtk(self._h, stage, kind, fmt, os.fsencode(path)), "erlbm_write_vtk")

    def run(self, n_steps: int, bc: dict | None = None, energy_every: int = 0, energy_factor: float = 2.0,
            density_check: bool = False, density_limit: float = 10.0) -> dict:
        b = _bc(bc)
        c = _lib.Checks(int(energy_every), float(energy_factor), int(bool(density_check)), float(density_limit))
        r = _lib.RunResult()
        check(lib().erlbm_run(self._h, int(n_steps), C.byref(b) if b is not None else None, C.byref(c), C.byref(r)),
              "erlbm_run")
        return dict(label=r.label, decided_step=r.decided_step, steps_done=r.steps_done, margin=r.margin)


def read_geo(path: str, pts_in: int = 0, pts_out: int = 0, wall: bool = True):
    """read_geo (LBM_functions.cpp:282-353): (nx, ny, nz, solid) of a legacy VTK geometry file, with
    fluid layers added in x; `solid` is the uint8 mask erlbm_desc takes (x fastest, 1 = solid)."""
    nx, ny, nz = C.c_int(), C.c_int(), C.c_int()
    p = os.fsencode(path)
    check(lib().erlbm_read_geo(p, pts_in, pts_out, int(wall), C.byref(nx), C.byref(ny), C.byref(nz), None, 0),
          "erlbm_read_geo")
    solid = np.zeros(nx.value * ny.value * nz.value, np.uint8)
    check(lib().erlbm_read_geo(p, pts_in, pts_out, int(wall), C.byref(nx), C.byref(ny), C.byref(nz), _dptr(solid),
                               solid.size), "erlbm_read_geo")
    return nx.value, ny.value, nz.value, solid


def velocity_error(sim: Lattice, ref: Lattice, text_digits: int = 0, sim_stage: int = STAGE_POST_COLLISION,
                   ref_stage: int = STAGE_POST_COLLISION):
    """tools/error_calculator.cpp between two lattices on the GPU: (E_vec, E_mod) of sim's velocity
    against ref's sampled at the same physical points.  text_digits = 6 reproduces the tool, which
    reads 6-significant-digit ASCII files; 0 uses the full-precision fields."""
    ev, em = C.c_double(), C.c_double()
    check(lib().erlbm_velocity_error(sim._h, sim_stage, ref._h, ref_stage, int(text_digits), C.byref(ev), C.byref(em)),
          "erlbm_velocity_error")
    return ev.value, em.value


def _bc(bc: dict | None):
    """erlbm_bc from a dict: inlet_x, u_in, outlet_x, rho_out, inlet_kind, parabolic_L, outlet_kind and
    open_y (-1 or absent = no open y plane)."""
    if bc is None:
        return None
    oy = int(bc.get("open_y", -1))
    return _lib.BC(int(bc.get("inlet_x", -1)), float(bc.get("u_in", 0.0)), int(bc.get("outlet_x", -1)),
                   float(bc.get("rho_out", 1.0)), int(bc.get("inlet_kind", 0)), int(bc.get("parabolic_L", 0)),
                   int(bc.get("outlet_kind", 0)), 1 if oy >= 0 else 0, max(oy, 0))


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


def fp64_rate() -> float:
    """FP64 add / multiply operations per second of the current GPU (erlbm_fp64_rate)."""
    v = C.c_double()
    check(lib().erlbm_fp64_rate(C.byref(v)), "erlbm_fp64_rate")
    return v.value


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


# ---- batched runs and stability maps --------------------------------------------------------------

def map_run(kind: int, points=None, precision: int = FP64, op: int = OP_EXTREG, tau_nh: float = 0.65, L: int = 16,
            ma: float = 0.1, n_i: int = 400, n_j: int = 400, max_steps: int = 0, slots: int = 0):
    """A stability map (or a subset of its points) in one batched launch.

    kind: MAP_TAYLOR_GREEN (main_stability-map_taylor-green.cpp) or MAP_OBSTACLE
    (main_stability-map_obstacle.cpp).  points: list of (i, j) map indices, or None for the whole
    n_i x n_j grid (i fastest).  op = 0 on the Taylor-Green map runs every point with RLBM and with
    E-RLBM (results concatenated, RLBM first).  slots: resident lattices per SM, 0 = as many as fit,
    -1 = the autotuner's cached choice.  Returns (labels, decided_step, margins) arrays.
    """
    if slots < 0:
        from . import autotune
        slots = autotune.best_slots(kind, precision)
    if points is None:
        n, pi, pj = n_i * n_j, None, None
    else:
        pi = np.ascontiguousarray([p[0] for p in points], dtype=np.int32)
        pj = np.ascontiguousarray([p[1] for p in points], dtype=np.int32)
        n = len(points)
    d = _lib.MapDesc(kind, precision, op, tau_nh, L, ma, n_i, n_j, 0 if points is None else n,
                     None if pi is None else pi.ctypes.data, None if pj is None else pj.ctypes.data, max_steps, slots)
    m = n * (2 if (kind == MAP_TAYLOR_GREEN and op == 0) else 1)
    labels = np.zeros(m, np.int32)
    dec = np.zeros(m, np.int32)
    mg = np.zeros(m, np.float64)
    check(lib().erlbm_map_run(C.byref(d), _dptr(labels), _dptr(dec), _dptr(mg)), "erlbm_map_run")
    return labels, dec, mg


def map_run_refined(kind: int, op: int = OP_EXTREG, tau_nh: float = 0.65, L: int = 16, ma: float = 0.1,
                    n_i: int = 400, n_j: int = 400, max_steps: int = 0, slots: int = 0, radius: int = 2,
                    late_fraction: float = 0.3, probe_stride: int = 16, max_passes: int = 0,
                    return_passes: bool = False):
    """A whole stability map screened in FP32-shifted, with the boundary points refined in FP64.

    Pass 1 runs again in FP64 (the reference's results) the points within `radius` map steps of an
    FP32 label change, the FP32 runs that turned unstable after `late_fraction` of their budget and
    the probe points (every `probe_stride`-th point in i and j, 0 = none); each further pass runs the
    FP32 points within `radius` of a label change of the map as it stands, until none is left (or
    `max_passes`, 0 = no cap).  Returns (labels, decided_step, margins, refined) with refined a boolean
    mask, and the number of FP64 passes after them when return_passes is set.
    """
    d = _lib.MapDesc(kind, FP32_SHIFTED, op, tau_nh, L, ma, n_i, n_j, 0, None, None, max_steps, slots)
    r = _lib.RefineDesc(radius, late_fraction, probe_stride, max_passes)
    m = n_i * n_j * (2 if (kind == MAP_TAYLOR_GREEN and op == 0) else 1)
    labels = np.zeros(m, np.int32)
    dec = np.zeros(m, np.int32)
    mg = np.zeros(m, np.float64)
    ref = np.zeros(m, np.uint8)
    passes = C.c_int(0)
    check(lib().erlbm_map_run_refined(C.byref(d), C.byref(r), _dptr(labels), _dptr(dec), _dptr(mg), _dptr(ref),
                                      C.byref(passes)), "erlbm_map_run_refined")
    if return_passes:
        return labels, dec, mg, ref.astype(bool), passes.value
    return labels, dec, mg, ref.astype(bool)


def batch_run(q: int, nx: int, ny: int, runs, precision: int = FP64, solid=None, inlet_x: int = -1,
              outlet_x: int = -1, rho0: float = 1.0, energy_every: int = 0, energy_factor: float = 2.0,
              density_check: bool = False, density_limit: float = 10.0, init: int = INIT_REST, aos=None,
              slots: int = 0):
    """Independent runs of one small geometry in one persistent launch.

    runs: iterable of dicts with op, tau, tau_nh, u0, n_steps and (for INIT_AOS) aos_offset.
    Returns a list of result dicts (label, decided_step, steps_done, status, margin, energy).
    """
    runs = list(runs)
    specs = (_lib.RunSpec * max(1, len(runs)))()
    for k, r in enumerate(runs):
        specs[k] = _lib.RunSpec(int(r.get("op", OP_EXTREG)), float(r["tau"]), float(r.get("tau_nh", 1.0)),
                                float(r.get("u0", 0.0)), int(r["n_steps"]), int(r.get("aos_offset", 0)))
    sol = None
    if solid is not None:
        sol = np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1)
    d = _lib.BatchDesc(q, nx, ny, None if sol is None else sol.ctypes.data, inlet_x, outlet_x, rho0, energy_every,
                       energy_factor, int(bool(density_check)), density_limit, init, precision, slots)
    a = None
    if aos is not None:
        a = np.ascontiguousarray(aos, dtype=np.float64).reshape(-1)
    out = (_lib.BatchResult * max(1, len(runs)))()
    check(lib().erlbm_batch_run(C.byref(d), len(runs), specs, None if a is None else a.ctypes.data,
                                0 if a is None else a.size, out), "erlbm_batch_run")
    return [dict(label=o.label, decided_step=o.decided_step, steps_done=o.steps_done, status=o.status,
                 margin=o.margin, energy=o.energy) for o in out[:len(runs)]]


# ---- request server ---------------------------------------------------------------------------------

class Server:
    """Continuous-batching server (erlbm_server_*): submit runs while others are on the GPU."""

    def __init__(self, hbm_budget_bytes: int = 8 << 30, slot_ctas: int = 0, max_streams: int = 0,
                 queue_capacity: int = 0, team_ctas: int = 0, team_max_nodes: int = 0, team_wait_us: int = 0):
        d = _lib.ServerDesc(int(hbm_budget_bytes), int(slot_ctas), int(max_streams), int(queue_capacity),
                            int(team_ctas), int(team_max_nodes), int(team_wait_us))
        h = C.c_void_p()
        check(lib().erlbm_server_start(C.byref(d), C.byref(h)), "erlbm_server_start")
        self._h = h

    def submit(self, kind: int, precision: int = FP64, op: int = OP_EXTREG, L: int = 16, sx: int = 1, sy: int = 1,
               tau: float = 0.6, tau_nh: float = 0.65, u0: float = 0.05, n_steps: int = 100) -> int:
        q = _lib.Request(kind, precision, op, L, sx, sy, tau, tau_nh, u0, n_steps)
        t = C.c_int64()
        check(lib().erlbm_server_submit(self._h, C.byref(q), C.byref(t)), "erlbm_server_submit")
        return t.value

    @staticmethod
    def _res(r):
        return dict(status=r.status, label=r.label, steps_done=r.steps_done, decided_step=r.decided_step,
                    energy=r.energy, margin=r.margin, t_submit=r.t_submit, t_admit=r.t_admit, t_done=r.t_done,
                    lane=r.lane)

    def poll(self, ticket: int):
        r = _lib.Result()
        rc = lib().erlbm_server_poll(self._h, ticket, C.byref(r))
        if rc == 1:
            return None
        check(rc, "erlbm_server_poll")
        return self._res(r)

    def wait(self, ticket: int, timeout: float = 600.0):
        r = _lib.Result()
        check(lib().erlbm_server_wait(self._h, ticket, C.byref(r), timeout), "erlbm_server_wait")
        return self._res(r)

    def clock(self) -> float:
        return lib().erlbm_server_clock(self._h)

    def stop(self):
        if getattr(self, "_h", None):
            check(lib().erlbm_server_stop(self._h), "erlbm_server_stop")
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.stop()
