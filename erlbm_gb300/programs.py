"""The double-shear-layer study of the reference (Figs. 4 and 5) run through the engine.

``double_shear_layer`` is main_double-shear-layer.cpp's loop: the initial field of
initial_double_shear_layer (:48-66), steps 0 .. n_steps - 1 with n_steps = round(t_final L / U0) + 1,
and every `interval` steps, on the post-collision populations of that step, the kinetic energy, the
stability check sqrt(2 E / n) > 0.4 (:187-203) and, optionally, the field files the program writes
(vel_<t*>.vtk, vor_<step>.vtk).  ``fig4_table`` is scripts/run_fig4_double_shear_layer.sh: an RLBM
reference run at L = 2048, the runs at L = 64 ... 1024 for each model, and tools/error_calculator's
E_vector and E_magnitude at t* = 1 for each, computed on the GPU from the resident fields.
"""
from __future__ import annotations

import math
import os

from . import (FIELD_VELOCITY, FIELD_VORTICITY, FP32_SHIFTED, FP64, OP_EXTREG, OP_REG, STAGE_POST_COLLISION,
               VTK_ASCII, Lattice, init_double_shear, velocity_error)

U0 = 1.0 / 32.0
U_LIMIT = 0.4  # main_double-shear-layer.cpp:41

# Fig. 4's models as the run script names them: (name, operator, tau_nh)
FIG4_MODELS = (("REG", OP_REG, 1.0), ("ERLBM065", OP_EXTREG, 0.65), ("ERLBM075", OP_EXTREG, 0.75))


def script_tau(L: int, Re: float = 80000.0) -> float:
    """tau as the run script passes it: 1/2 + 3 U0 L / Re printed with %.12g and read back (--tau)."""
    return float("%.12g" % (0.5 + 3.0 * (1.0 / 32.0) * L / Re))


def double_shear_layer(L: int, op: int, tau: float, tau_nh: float = 0.65, t_final: float = 1.0,
                       dt_out: float = 1.0 / 16.0, precision: int = FP64, out_dir: str | None = None,
                       vorticity: bool = False, fmt: int = VTK_ASCII):
    """Runs the program to t_final and returns (lattice, record).  The lattice holds the post-collision
    populations of the last step; record lists (t*, E) per output and the step that stopped an
    unstable run (None if it ran to the end).  tau_nh is used by E-RLBM only (RLBM fixes it to 1)."""
    per_t = int(round(L / U0))
    n_steps = int(round(t_final * per_t)) + 1
    interval = max(1, int(round(dt_out * per_t)))
    lat = Lattice(9, L, L, 1, None, tau, 1.0 if op == OP_REG else tau_nh, op, precision)
    if precision == FP32_SHIFTED and L % 128 == 0:
        from . import autotune  # the measured launch shape (two steps per launch on GB300), cached per device
        autotune.apply_periodic(lat)
    lat.set_populations(init_double_shear(L))
    n = L * L
    rec = {"energy": [], "unstable_step": None, "n_steps": n_steps, "interval": interval}
    done = 0
    for s in range(0, n_steps, interval):
        lat.step(s + 1 - done)  # through the collision of step s
        done = s + 1
        t_adm = s * U0 / L
        e = lat.kinetic_energy(STAGE_POST_COLLISION)
        rec["energy"].append((t_adm, e))
        if not math.isfinite(e) or math.sqrt(2.0 * e / n) > U_LIMIT:
            rec["unstable_step"] = s
            return lat, rec
        if out_dir is not None:
            lat.write_vtk(os.path.join(out_dir, "vel_%f.vtk" % t_adm), FIELD_VELOCITY, fmt)
            if vorticity:
                lat.write_vtk(os.path.join(out_dir, "vor_%d.vtk" % s), FIELD_VORTICITY, fmt)
    if done < n_steps:
        lat.step(n_steps - done)
    return lat, rec


def fig4_table(Ls=(64, 128, 256, 512, 1024), L_ref: int = 2048, models=FIG4_MODELS, precision: int = FP64,
               text_digits: int = 6, log=None):
    """E_vector and E_magnitude at t* = 1 of each model and L against the RLBM run at L_ref, as
    scripts/run_fig4_double_shear_layer.sh and tools/error_calculator compute them (text_digits = 6:
    the tool's 6-digit ASCII inputs; 0: full precision).  Rows: dict(model, L, tau, tau_nh, E_vector,
    E_magnitude)."""
    ref, _ = double_shear_layer(L_ref, OP_REG, script_tau(L_ref), 1.0, 1.0, precision=precision)
    rows = []
    with ref:
        for L in Ls:
            for name, op, tnh in models:
                sim, r = double_shear_layer(L, op, script_tau(L), tnh, 1.0, precision=precision)
                with sim:
                    ev, em = (math.nan, math.nan) if r["unstable_step"] is not None else \
                        velocity_error(sim, ref, text_digits)
                rows.append(dict(model=name, L=L, tau=script_tau(L), tau_nh=tnh, E_vector=ev, E_magnitude=em))
                if log:
                    log(rows[-1])
    return rows


def precision_error(L: int, t_stars=(0.125, 0.25, 0.5, 1.0), precision: int = FP32_SHIFTED, op: int = OP_EXTREG,
                    tau_nh: float = 0.65, log=None):
    """The double shear layer of main_double-shear-layer.cpp (Re = 80000, U0 = 1/32) run in `precision`
    and in FP64 (the reference's results) from the same initial populations: the relative L2 error of
    the post-collision velocity of step 32 L t*, ||u - u64|| / ||u64|| over all nodes (the formula of
    tools/error_calculator.cpp:88-105, in memory), for each t*.  Returns {t*: error}."""
    import numpy as np
    tau = 0.5 + 3.0 * U0 * L / 80000.0
    tnh = 1.0 if op == OP_REG else tau_nh
    f0 = init_double_shear(L)
    out = {}
    with Lattice(9, L, L, 1, None, tau, tnh, op, FP64) as l64, Lattice(9, L, L, 1, None, tau, tnh, op,
                                                                        precision) as lp:
        if precision == FP32_SHIFTED and L % 128 == 0:
            from . import autotune
            autotune.apply_periodic(lp)
        l64.set_populations(f0)
        lp.set_populations(f0)
        done = 0
        for t in sorted(t_stars):
            s = int(round(t * L / U0))
            l64.step(s + 1 - done)
            lp.step(s + 1 - done)
            done = s + 1
            _, u64 = l64.macroscopic(STAGE_POST_COLLISION)
            _, up = lp.macroscopic(STAGE_POST_COLLISION)
            out[t] = float(np.linalg.norm(up - u64) / np.linalg.norm(u64))
            if log:
                log(L, t, out[t])
    return out
