"""ctypes bindings of the CPU oracle -- TEST INFRASTRUCTURE, NOT THE PRODUCT.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module, as the
checker or as the timed CPU baseline.  ``load()`` builds ``liberlbm_oracle.so`` with the Makefile
beside it when needed.  ``load_ref(q)`` opens the reference library compiled from its own sources
(``_ref/libref_d*.so``), which exists only where the reference tree was available at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OP_BGK, OP_MRT, OP_REG, OP_EXTREG = 1, 2, 3, 4

_lib = None
_ref = {}

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


class OrcBC(C.Structure):
    _fields_ = [("inlet_x", C.c_int), ("u_in", C.c_double), ("outlet_x", C.c_int), ("rho_out", C.c_double),
                ("inlet_kind", C.c_int), ("parabolic_L", C.c_int), ("outlet_kind", C.c_int), ("open_y", C.c_int)]


INLET_ZOUHE, INLET_PARABOLIC = 0, 1
OUTLET_DENSITY, OUTLET_OPEN, OUTLET_CONVECTIVE = 0, 1, 2


def orc_bc(bc: dict) -> OrcBC:
    return OrcBC(bc.get("inlet_x", -1), bc.get("u_in", 0.0), bc.get("outlet_x", -1), bc.get("rho_out", 1.0),
                 bc.get("inlet_kind", 0), bc.get("parabolic_L", 0), bc.get("outlet_kind", 0), bc.get("open_y", -1))


def build(force: bool = False) -> str:
    so = os.path.join(HERE, "liberlbm_oracle.so")
    srcs = [os.path.join(HERE, f) for f in ("erlbm_oracle.c", "fp32_shifted.c", "erlbm_oracle.h")]
    if force or not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(f) for f in srcs):
        subprocess.run(["make", "-s", "-C", HERE, "liberlbm_oracle.so"], check=True)
    return so


def load():
    global _lib
    if _lib is not None:
        return _lib
    lib = C.CDLL(build())
    vp = C.c_void_p
    sig = {
        "orc_create": (vp, [C.c_int, C.c_int, C.c_int, C.c_int, vp, C.c_double, C.c_double, C.c_int]),
        "orc_destroy": (None, [vp]),
        "orc_fluid_count": (C.c_int, [vp]),
        "orc_set_params": (None, [vp, C.c_double, C.c_double, C.c_int]),
        "orc_set_populations": (None, [vp, _dp]),
        "orc_get_populations": (None, [vp, _dp, C.c_int]),
        "orc_step": (None, [vp, C.c_int, vp, C.c_int]),
        "orc_kinetic_energy": (C.c_double, [vp, C.c_int]),
        "orc_max_abs_density": (C.c_double, [vp, C.c_int, C.POINTER(C.c_int)]),
        "orc_equilibrium": (None, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _dp]),
        "orc_collide_site": (None, [C.c_int, _dp, C.c_int, C.c_double, C.c_double]),
        "orc_init_taylor_green": (None, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int,
                                         C.c_int, _dp]),
        "orc_taylor_green_error": (None, [C.c_int, C.c_int, _dp, C.c_double, C.c_double, C.c_int, C.c_int, _dp]),
        "orc_taylor_green_program": (None, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                            C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, _dp]),
        "orc_init_double_shear": (None, [C.c_int, C.c_double, _dp]),
        "orc_tg_map_params": (None, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                     C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "orc_obstacle_map_params": (None, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                           C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "orc_tg_map_point": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                       C.POINTER(C.c_int), C.POINTER(C.c_double)]),
        "orc_obstacle_geometry": (None, [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), vp]),
        "orc_obstacle_map_point": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                             C.POINTER(C.c_int), C.POINTER(C.c_double)]),
        "orc_tg_map": (None, [C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, _ip, _ip, C.c_int,
                              C.c_int, _ip, _ip, _dp]),
        "orc_obstacle_map": (None, [C.c_int, C.c_int, C.c_double, C.c_int, _ip, _ip, C.c_int, C.c_int,
                                    _ip, _ip, _dp]),
        "orc_max_threads": (C.c_int, []),
        "orc_field": (None, [C.c_int, C.c_int, C.c_int, C.c_int, vp, _dp, C.c_int, _dp]),
        "orc_read_geo": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int), vp]),
        "orc_write_vtk": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, vp, _dp, C.c_int, C.c_int, C.c_char_p]),
        "orc_velocity_error": (C.c_int, [C.c_int, C.c_int, _dp, C.c_int, C.c_int, _dp, C.c_int,
                                         C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class Lattice:
    """One lattice of the oracle: AoS populations in fluid-index order, push streaming."""

    def __init__(self, q, nx, ny, nz=1, solid=None, tau=0.6, tau_nh=0.65, op=OP_EXTREG):
        lib = load()
        self.q, self.nx, self.ny, self.nz = q, nx, ny, nz
        self._solid = None if solid is None else np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1)
        sp = None if self._solid is None else self._solid.ctypes.data
        self.h = lib.orc_create(q, nx, ny, nz, sp, tau, tau_nh, op)
        if not self.h:
            raise ValueError("oracle: invalid lattice")
        self.n_fluid = lib.orc_fluid_count(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            load().orc_destroy(self.h)
            self.h = None

    def set_params(self, tau, tau_nh, op):
        load().orc_set_params(self.h, tau, tau_nh, op)

    def set(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        assert f.size == self.n_fluid * self.q
        load().orc_set_populations(self.h, f)

    def get(self, stage=0):
        out = np.empty(self.n_fluid * self.q, dtype=np.float64)
        load().orc_get_populations(self.h, out, stage)
        return out

    def step(self, n, bc=None, threads=1):
        b = None
        if bc is not None:
            b = C.byref(orc_bc(bc))
        load().orc_step(self.h, int(n), b, int(threads))

    def kinetic_energy(self, stage=0):
        return load().orc_kinetic_energy(self.h, stage)

    def max_abs_density(self, stage=0):
        nf = C.c_int(0)
        m = load().orc_max_abs_density(self.h, stage, C.byref(nf))
        return m, bool(nf.value)


def equilibrium(q, ux, uy, uz, rho):
    out = np.empty(q)
    load().orc_equilibrium(q, ux, uy, uz, rho, out)
    return out


def init_taylor_green(q, L, u0, tau, poisson=True, neq=True, variant=0, nz=1):
    out = np.empty(L * L * nz * q)
    load().orc_init_taylor_green(q, L, nz, u0, tau, int(poisson), int(neq), int(variant), out)
    return out


def taylor_green_error(q, L, f, u0, visc, step, variant=0):
    out = np.empty(3)
    load().orc_taylor_green_error(q, L, np.ascontiguousarray(f, dtype=np.float64), u0, visc, step, variant, out)
    return out


def taylor_green_program(L, op, tau_nh=0.65, Re=50.0, u0=0.0, tau=None, neq=True, poisson=True, variant=0,
                         q=9, threads=0):
    out = np.empty(7)
    threads = threads or load().orc_max_threads()
    load().orc_taylor_green_program(q, L, op, tau_nh, Re, u0, int(tau is not None), tau or 0.0, int(neq),
                                    int(poisson), int(variant), threads, out)
    return dict(tau=out[0], tau_nh=out[1], u0=out[2], steps=int(out[3]), e_vec=out[4], e_mag=out[5],
                nu_rel=out[6])


def init_double_shear(L, rho=1.0):
    out = np.empty(L * L * 9)
    load().orc_init_double_shear(L, rho, out)
    return out


def tg_map_params(i, j, n_ma, n_nu, op, tau_nh):
    a, b, c = C.c_double(), C.c_double(), C.c_double()
    load().orc_tg_map_params(i, j, n_ma, n_nu, op, tau_nh, C.byref(a), C.byref(b), C.byref(c))
    return a.value, b.value, c.value  # u0, tau, tau_nh


def obstacle_map_params(i, j, n_tau, n_nu, ma=0.1):
    a, b, c = C.c_double(), C.c_double(), C.c_double()
    load().orc_obstacle_map_params(i, j, n_tau, n_nu, ma, C.byref(a), C.byref(b), C.byref(c))
    return a.value, b.value, c.value  # u_imp, tau, tau_nh


def tg_map_point(L, op, tau, tau_nh, u0, max_steps=0):
    ds, mg = C.c_int(), C.c_double()
    lab = load().orc_tg_map_point(L, op, tau, tau_nh, u0, max_steps, C.byref(ds), C.byref(mg))
    return lab, ds.value, mg.value


def obstacle_geometry(sx=1, sy=1):
    nx, ny = C.c_int(), C.c_int()
    load().orc_obstacle_geometry(sx, sy, C.byref(nx), C.byref(ny), None)
    solid = np.zeros(nx.value * ny.value, dtype=np.uint8)
    load().orc_obstacle_geometry(sx, sy, C.byref(nx), C.byref(ny), solid.ctypes.data)
    return nx.value, ny.value, solid


def obstacle_map_point(tau, tau_nh, u_imp, sx=1, sy=1, max_steps=0):
    ds, mg = C.c_int(), C.c_double()
    lab = load().orc_obstacle_map_point(sx, sy, tau, tau_nh, u_imp, max_steps, C.byref(ds), C.byref(mg))
    return lab, ds.value, mg.value


def tg_map(points, L=16, op=OP_EXTREG, tau_nh=0.65, n_ma=400, n_nu=400, max_steps=0, threads=0):
    pi = np.ascontiguousarray([p[0] for p in points], dtype=np.int32)
    pj = np.ascontiguousarray([p[1] for p in points], dtype=np.int32)
    n = len(points)
    lab, dec, mg = np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n, np.float64)
    threads = threads or load().orc_max_threads()
    load().orc_tg_map(L, op, tau_nh, n_ma, n_nu, n, pi, pj, max_steps, threads, lab, dec, mg)
    return lab, dec, mg


def obstacle_map(points, n_tau=400, n_nu=400, ma=0.1, max_steps=0, threads=0):
    pi = np.ascontiguousarray([p[0] for p in points], dtype=np.int32)
    pj = np.ascontiguousarray([p[1] for p in points], dtype=np.int32)
    n = len(points)
    lab, dec, mg = np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n, np.float64)
    threads = threads or load().orc_max_threads()
    load().orc_obstacle_map(n_tau, n_nu, ma, n, pi, pj, max_steps, threads, lab, dec, mg)
    return lab, dec, mg


FIELD_VELOCITY, FIELD_VORTICITY, FIELD_DENSITY = 1, 2, 3
VTK_ASCII, VTK_BINARY_FLOAT, VTK_BINARY_DOUBLE = 0, 1, 2


def _solid_ptr(solid):
    if solid is None:
        return None, None
    s = np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1)
    return s, s.ctypes.data


def field(q, nx, ny, nz, solid, aos, kind):
    """The rec_* writers' field at every box node (x fastest, solid nodes 0): velocity or vorticity
    (3 values per node) or density."""
    s, sp = _solid_ptr(solid)
    n = nx * ny * nz * (1 if kind == FIELD_DENSITY else 3)
    out = np.empty(n)
    load().orc_field(q, nx, ny, nz, sp, np.ascontiguousarray(aos, dtype=np.float64), kind, out)
    return out


def write_vtk(q, nx, ny, nz, solid, aos, kind, fmt, path):
    s, sp = _solid_ptr(solid)
    rc = load().orc_write_vtk(q, nx, ny, nz, sp, np.ascontiguousarray(aos, dtype=np.float64), kind, fmt,
                              os.fsencode(path))
    if rc:
        raise OSError(f"cannot write {path}")


def fp32_periodic_d2q9(nx, ny, op, tau, tau_nh, f_in, n_steps):
    """The engine's FP32-shifted D2Q9 periodic update restated on the CPU (fp32_shifted.c): the
    post-collision populations after n_steps steps, the first colliding in place."""
    f_in = np.ascontiguousarray(f_in, dtype=np.float64)
    out = np.empty_like(f_in)
    fn = load().orc32_periodic_d2q9
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _dp, C.c_int, _dp]
    if fn(nx, ny, op, tau, tau_nh, f_in, n_steps, out):
        raise ValueError("orc32_periodic_d2q9: bad arguments")
    return out


def fp32_periodic_solid(q, nx, ny, nz, solid, op, tau, tau_nh, f_in, n_steps):
    """The restatement with a solid mask (halfway bounce-back): f_in and the result hold every node of
    the box in x-fastest order; solid nodes are left as given."""
    f_in = np.ascontiguousarray(f_in, dtype=np.float64)
    out = np.empty_like(f_in)
    fn = load().orc32_periodic_solid
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_double, C.c_double, _dp, C.c_int,
                   _dp]
    sp = None
    if solid is not None:
        solid = np.ascontiguousarray(solid, dtype=np.uint8)
        if solid.size != nx * ny * nz:
            raise ValueError("solid mask size")
        sp = solid.ctypes.data
    if f_in.size != nx * ny * nz * q or fn(q, nx, ny, nz, sp, op, tau, tau_nh, f_in, n_steps, out):
        raise ValueError("orc32_periodic_solid: bad arguments")
    return out


def fp32_channel(q, nx, ny, nz, solid, op, tau, tau_nh, f_in, n_steps, inlet_x=-1, u_in=0.0, outlet_x=-1,
                 rho_out=1.0, outlet_kind=0, open_y=-1, inlet_kind=0, parabolic_L=0):
    """The restatement with a solid mask and boundary planes: a velocity inlet at inlet_x, Zou-He
    (inlet_kind 0) or parabolic with a channel width of parabolic_L fluid nodes (1); an outlet at
    outlet_x of kind 0 (density, devnull_rho_x), 1 (open, D2Q9) or 2 (convective); the D2Q9 open y
    plane open_y.  f_in and the result hold every node of the box."""
    f_in = np.ascontiguousarray(f_in, dtype=np.float64)
    out = np.empty_like(f_in)
    fn = load().orc32_channel_ex
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int,
                   C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, _dp, C.c_int, _dp]
    sp = None
    if solid is not None:
        solid = np.ascontiguousarray(solid, dtype=np.uint8)
        if solid.size != nx * ny * nz:
            raise ValueError("solid mask size")
        sp = solid.ctypes.data
    if f_in.size != nx * ny * nz * q or fn(q, nx, ny, nz, sp, op, tau, tau_nh, inlet_x, u_in, inlet_kind, parabolic_L,
                                           outlet_x, outlet_kind, rho_out, open_y, f_in, n_steps, out):
        raise ValueError("orc32_channel_ex: bad arguments")
    return out


def fp32_pair_periodic_d2q9(nx, ny, op, tau, tau_nh, f_in, n_steps):
    """The compensated FP32 form (float-pair populations) restated on the CPU, periodic D2Q9: n_steps
    steps from the post-stream populations f_in (the first colliding in place); the post-collision
    populations f = w + hi + lo."""
    f_in = np.ascontiguousarray(f_in, dtype=np.float64)
    out = np.empty_like(f_in)
    fn = load().orc32p_periodic_d2q9
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _dp, C.c_int, _dp]
    if f_in.size != nx * ny * 9 or fn(nx, ny, op, tau, tau_nh, f_in, n_steps, out):
        raise ValueError("orc32p_periodic_d2q9: bad arguments")
    return out


def fp32_batch_run(q, nx, ny, op, tau, tau_nh, u0, n_steps, block, npt, solid=None, inlet_x=-1, outlet_x=-1,
                   rho0=1.0, energy_every=0, energy_factor=2.0, density_check=False, density_limit=10.0, init=0):
    """One run of the engine's batched FP32 map kernel restated bit for bit (orc32_batch_run): the CTA
    shape (block threads, npt nodes each) fixes the energy sum's order.  Returns the result fields."""
    fn = load().orc32_batch_run
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int,
                   C.c_double, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int,
                   C.c_void_p, C.c_void_p]
    sp = None
    if solid is not None:
        solid = np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1)
        sp = solid.ctypes.data
    o4, o2 = np.zeros(4, np.int32), np.zeros(2, np.float64)
    if fn(q, nx, ny, sp, inlet_x, outlet_x, rho0, energy_every, energy_factor, int(bool(density_check)),
          density_limit, init, op, tau, tau_nh, u0, n_steps, block, npt, o4.ctypes.data, o2.ctypes.data):
        raise ValueError("orc32_batch_run: bad arguments")
    return dict(label=int(o4[0]), decided_step=int(o4[1]), steps_done=int(o4[2]), status=int(o4[3]),
                margin=float(o2[0]), energy=float(o2[1]))


def fp32_periodic_d3q19(nx, ny, nz, op, tau, tau_nh, f_in, n_steps):
    """The same restatement for D3Q19 (BGK, RLBM, E-RLBM) on an nx x ny x nz periodic box."""
    f_in = np.ascontiguousarray(f_in, dtype=np.float64)
    out = np.empty_like(f_in)
    fn = load().orc32_periodic_d3q19
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _dp, C.c_int, _dp]
    if fn(nx, ny, nz, op, tau, tau_nh, f_in, n_steps, out):
        raise ValueError("orc32_periodic_d3q19: bad arguments")
    return out


def read_geo(path, pts_in=0, pts_out=0, wall=True):
    """read_geo's solid mask: (nx, ny, nz, solid uint8 array, fluid count)."""
    nx, ny, nz = C.c_int(), C.c_int(), C.c_int()
    n = load().orc_read_geo(os.fsencode(path), pts_in, pts_out, int(wall), C.byref(nx), C.byref(ny), C.byref(nz), None)
    if n < 0:
        raise OSError(f"cannot read {path}")
    solid = np.zeros(nx.value * ny.value * nz.value, np.uint8)
    n = load().orc_read_geo(os.fsencode(path), pts_in, pts_out, int(wall), C.byref(nx), C.byref(ny), C.byref(nz),
                            solid.ctypes.data)
    return nx.value, ny.value, nz.value, solid, n


def velocity_error(nx, ny, vel, nx_ref, ny_ref, vel_ref, text_digits=0):
    """tools/error_calculator.cpp on two velocity fields (3 values per node); returns (E_vec, E_mod)."""
    ev, em = C.c_double(), C.c_double()
    rc = load().orc_velocity_error(nx, ny, np.ascontiguousarray(vel, dtype=np.float64), nx_ref, ny_ref,
                                   np.ascontiguousarray(vel_ref, dtype=np.float64), text_digits, C.byref(ev),
                                   C.byref(em))
    if rc:
        raise ValueError("the reference grid must refine the simulation grid by one integer factor")
    return ev.value, em.value


# ---------------------------------------------------------------------------------------------
# The reference library compiled from its own sources (present only where it could be built)
# ---------------------------------------------------------------------------------------------

def ref_available(q: int) -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", f"libref_d{'2q9' if q == 9 else '3q19'}.so"))


def load_ref(q: int):
    if q in _ref:
        return _ref[q]
    path = os.path.join(HERE, "_ref", f"libref_d{'2q9' if q == 9 else '3q19'}.so")
    lib = C.CDLL(path)
    p = f"ref{q}_"
    vp = C.c_void_p
    getattr(lib, p + "run").restype = C.c_int
    getattr(lib, p + "run").argtypes = [C.c_int, C.c_int, C.c_int, vp, C.c_int, C.c_double, C.c_double, _dp,
                                       C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, vp, vp, vp]
    getattr(lib, p + "run_bc").restype = C.c_int
    getattr(lib, p + "run_bc").argtypes = [C.c_int, C.c_int, C.c_int, vp, C.c_int, C.c_double, C.c_double, vp, C.c_int,
                                          vp, vp, vp, vp]
    getattr(lib, p + "read_geo").restype = C.c_int
    getattr(lib, p + "read_geo").argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]
    if q == 9:
        lib.ref9_init_taylor_green.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, _dp]
        lib.ref9_init_double_shear.argtypes = [C.c_int, C.c_double, _dp]
        lib.ref9_taylor_green_main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        lib.ref9_rec_field.argtypes = [C.c_int, C.c_int, C.c_int, vp, _dp, C.c_int, C.c_int, C.c_double, C.c_uint]
    else:
        lib.ref19_tg_map_point.restype = C.c_int
        lib.ref19_tg_map_point.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double]
        lib.ref19_obstacle_map_point.restype = C.c_int
        lib.ref19_obstacle_map_point.argtypes = [C.c_double, C.c_double, C.c_double]
        lib.ref19_rec_field.argtypes = [C.c_int, C.c_int, C.c_int, vp, _dp, C.c_int, C.c_int, C.c_double, C.c_uint]
    _ref[q] = lib
    return lib


def ref_run(q, nx, ny, nz, solid, op, tau, tau_nh, f_in, n_steps, inlet_x=-1, u_in=0.0, outlet_x=-1,
            rho_out=1.0):
    lib = load_ref(q)
    f_in = np.ascontiguousarray(f_in, dtype=np.float64)
    ps, pc, e = np.empty_like(f_in), np.empty_like(f_in), C.c_double()
    s = None
    if solid is not None:
        solid = np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1)
        s = solid.ctypes.data
    getattr(lib, f"ref{q}_run")(nx, ny, nz, s, op, tau, tau_nh, f_in, n_steps, inlet_x, u_in, outlet_x, rho_out,
                                ps.ctypes.data, pc.ctypes.data, C.addressof(e))
    return ps, pc, e.value
