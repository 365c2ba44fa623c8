"""Generates the golden fixtures in this folder.  Run where the reference tree is present:

    python tests/golden/make_golden.py [--reference PATH]

PATH defaults to $ERLBM_REFERENCE, else a "reference" directory beside the repository.

It reads the reference's published tables (data/*.csv, data/*.vtk) and runs the reference's own
library and program functions, compiled from their sources by oracle/Makefile (target `ref`), to
produce:

  published.json          Fig. 3 / feq-init / kappa_4 / Fig. 4 tables (numbers as published), the
                          unstable-point counts of the three published 400 x 400 maps, and their
                          20 x 20 subsamples at the README's indices (README "Previous version of
                          the code": TG i' = 20(i+1)-1, j' = 20 j; obstacle i' = 20 i, j' = 20 j).
  reference_maps_20x20.json
                          the same 20 x 20 subsamples computed by the reference's roda_ponto
                          (main_stability-map_taylor-green.cpp:41-104, main_stability-map_obstacle.cpp:75-123).
  reference_vectors.npz   inputs and outputs of short runs of the reference library (colisao_sitio +
                          propag_site loop with its boundary functions): small D2Q9 / D3Q19 lattices
                          under BGK, MRT (D2Q9), RLBM and E-RLBM, the obstacle channel, the
                          Taylor-Green and double-shear-layer initial fields.  --vectors-only rewrites
                          this file alone.
"""
from __future__ import annotations

import argparse
import ctypes as C
import hashlib
import json
import multiprocessing as mp
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def read_csv(path):
    lines = [l.strip() for l in open(path) if l.strip()]
    head = lines[0].split(",")
    rows = []
    for l in lines[1:]:
        vals = l.split(",")
        row = {}
        for h, v in zip(head, vals):
            try:
                row[h] = float(v) if any(c in v for c in ".e") or v.lstrip("-").isdigit() else v
            except ValueError:
                row[h] = v
        rows.append(row)
    return rows


def read_map(path):
    lines = open(path).read().split("\n")
    nx, ny = [int(v) for v in next(l for l in lines if l.startswith("DIMENSIONS")).split()[1:3]]
    k = next(n for n, l in enumerate(lines) if l.startswith("LOOKUP_TABLE"))
    vals = np.array(" ".join(lines[k + 1:]).split(), dtype=float)
    return vals[: nx * ny].reshape(ny, nx).astype(int)


TG_SUB = [(20 * (i + 1) - 1, 20 * j) for j in range(20) for i in range(20)]

# channel-boundary cases: (q, nx, ny, nz, walls at y = 0 and ny - 1 (else only at ny - 1), bc)
BC_CASES = (
    (9, 16, 10, 1, True, dict(inlet_x=1, inlet_kind=0, u_in=0.04, outlet_x=14, outlet_kind=0, rho_out=1.0)),
    (9, 16, 10, 1, True, dict(inlet_x=1, inlet_kind=1, parabolic_L=8, u_in=0.06, outlet_x=14, outlet_kind=1)),
    (9, 16, 10, 1, True, dict(inlet_x=1, inlet_kind=0, u_in=0.04, outlet_x=14, outlet_kind=2)),
    (9, 16, 10, 1, False, dict(inlet_x=1, inlet_kind=1, parabolic_L=9, u_in=0.05, outlet_x=14, outlet_kind=1,
                               open_y=0)),
    (19, 12, 8, 2, True, dict(inlet_x=1, inlet_kind=1, parabolic_L=6, u_in=0.05, outlet_x=10, outlet_kind=0,
                              rho_out=1.0)),
    (19, 12, 8, 2, True, dict(inlet_x=1, inlet_kind=0, u_in=0.04, outlet_x=10, outlet_kind=2)),
)


def channel_mask(nx, ny, nz, walls_y):
    """Solid planes x = 0 and x = nx - 1, and y = 0 and y = ny - 1 (walls_y) or y = ny - 1 alone."""
    s = np.zeros((nz, ny, nx), np.uint8)
    s[:, :, 0] = 1
    s[:, :, nx - 1] = 1
    s[:, ny - 1, :] = 1
    if walls_y:
        s[:, 0, :] = 1
    return s.reshape(-1)
OB_SUB = [(20 * i, 20 * j) for j in range(20) for i in range(20)]


def _worker_init():
    # the reference's boundary functions carry "omp parallel for" pragmas that its map programs
    # serialise with omp_set_max_active_levels(1) (main_stability-map_obstacle.cpp:137); one thread
    # per worker process does the same here
    os.environ["OMP_NUM_THREADS"] = "1"


def _ref_tg_point(args):
    i, j, op, tau_nh, n = args
    from oracle import oracle as O
    lib = O.load_ref(19)
    u0, tau, tnh = O.tg_map_params(i, j, n, n, op, tau_nh)
    return int(lib.ref19_tg_map_point(16, op, tau, tnh, u0))


def _ref_ob_point(args):
    i, j, n = args
    from oracle import oracle as O
    lib = O.load_ref(19)
    u, tau, tnh = O.obstacle_map_params(i, j, n, n, 0.1)
    return int(lib.ref19_obstacle_map_point(tau, tnh, u))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("ERLBM_REFERENCE")
                    or os.path.join(os.path.dirname(os.path.realpath(ROOT)), "reference"))
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--vectors-only", action="store_true", help="rewrite reference_vectors.npz only")
    a = ap.parse_args()
    ref = a.reference
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all", "ref", f"REFERENCE={ref}"], check=True)
    if not a.vectors_only:
        tables_and_maps(a)
    vectors()


def tables_and_maps(a):
    ref = a.reference
    from oracle import oracle as O

    # ---- published tables and maps -------------------------------------------------------------
    pub = {
        "fig3_taylor_green_Re50": read_csv(os.path.join(ref, "data", "fig3_taylor_green_Re50.csv")),
        "fig3_taylor_green_Re50_feq_init": read_csv(os.path.join(ref, "data", "fig3_taylor_green_Re50_feq_init.csv")),
        "kappa4_check_L64": read_csv(os.path.join(ref, "data", "kappa4_check_L64.csv")),
        "fig4_double_shear_Re80000": read_csv(os.path.join(ref, "data", "fig4_double_shear_Re80000.csv")),
        "maps": {},
    }
    for name, sub in (("fig1_map_reg", TG_SUB), ("fig1_map_erlbm065", TG_SUB), ("fig2_map_obstacle", OB_SUB)):
        m = read_map(os.path.join(ref, "data", name + ".vtk"))
        pub["maps"][name] = {"unstable": int(m.sum()), "points": 160000,
                             "subsample_20x20": [int(m[j, i]) for (i, j) in sub]}
    with open(os.path.join(HERE, "published.json"), "w") as f:
        json.dump(pub, f, indent=0)

    # ---- reference maps on the 20 x 20 subsample --------------------------------------------------
    ctx = mp.get_context("spawn")
    # grid400: the 400 x 400 map's own parameters at the subsampled indices;
    # grid20:  a 20 x 20 run (--n-ma 20 --n-nu 20, --n-tau 20), the README's quick-test protocol, whose
    #          axis values land on the same points up to the rounding of the axis formulas
    g20 = [(i, j) for j in range(20) for i in range(20)]
    with ctx.Pool(a.jobs, initializer=_worker_init) as pool:
        reg = pool.map(_ref_tg_point, [(i, j, O.OP_REG, 1.0, 400) for (i, j) in TG_SUB])
        erl = pool.map(_ref_tg_point, [(i, j, O.OP_EXTREG, 0.65, 400) for (i, j) in TG_SUB])
        obs = pool.map(_ref_ob_point, [(i, j, 400) for (i, j) in OB_SUB])
        reg20 = pool.map(_ref_tg_point, [(i, j, O.OP_REG, 1.0, 20) for (i, j) in g20])
        erl20 = pool.map(_ref_tg_point, [(i, j, O.OP_EXTREG, 0.65, 20) for (i, j) in g20])
        obs20 = pool.map(_ref_ob_point, [(i, j, 20) for (i, j) in g20])
    maps = {"tg_points": TG_SUB, "obstacle_points": OB_SUB, "tg_reg": reg, "tg_erlbm065": erl, "obstacle": obs,
            "grid20_points": g20, "grid20_tg_reg": reg20, "grid20_tg_erlbm065": erl20, "grid20_obstacle": obs20}
    with open(os.path.join(HERE, "reference_maps_20x20.json"), "w") as f:
        json.dump(maps, f)
    for name, lab, lab20 in (("fig1_map_reg", reg, reg20), ("fig1_map_erlbm065", erl, erl20),
                             ("fig2_map_obstacle", obs, obs20)):
        pubsub = np.array(pub["maps"][name]["subsample_20x20"])
        print(f"{name}: reference vs published subsample differ at {int(np.sum(np.array(lab) != pubsub))} "
              f"(400-grid parameters) and {int(np.sum(np.array(lab20) != pubsub))} (20 x 20 run) of 400 points")



def vectors():
    """Short runs of the reference library (colisao_sitio + propag_site loop with its boundary functions)."""
    from oracle import oracle as O
    rng = np.random.default_rng(20261203)
    vec = {}

    def near_eq(q, n, amp=0.05, noise=1e-3):
        fs = []
        for _ in range(n):
            u = rng.normal(0, amp, 3)
            if q == 9:
                u[2] = 0.0
            fs.append(O.equilibrium(q, u[0], u[1], u[2], 1 + rng.normal(0, 0.01)))
        f = np.concatenate(fs)
        return f + rng.normal(0, noise, f.size)

    for q, (nx, ny, nz), steps in ((9, (7, 5, 1), 13), (19, (6, 5, 3), 9)):
        f0 = near_eq(q, nx * ny * nz)
        # coll_MRT (op 2) exists for D2Q9 only (src/erlbm_common.h:74-76)
        for op, tnh in ((1, 0.57), (2, 0.57), (3, 1.0), (4, 0.65)) if q == 9 else ((1, 0.57), (3, 1.0), (4, 0.65)):
            ps, pc, e = O.ref_run(q, nx, ny, nz, None, op, 0.57, tnh, f0, steps)
            key = f"periodic_q{q}_op{op}"
            vec[key + "_in"] = f0
            vec[key + "_post_stream"] = ps
            vec[key + "_post_collision"] = pc
            vec[key + "_energy"] = np.array([e])
            vec[key + "_meta"] = np.array([nx, ny, nz, steps, op, 0.57, tnh])
    nx, ny, solid = O.obstacle_geometry()
    n_fluid = int((solid == 0).sum())
    f0 = np.tile(O.equilibrium(19, 0, 0, 0, 1.0), n_fluid)
    u = 0.1 / np.sqrt(3.0)
    ps, pc, e = O.ref_run(19, nx, ny, 1, solid, 4, 0.52, 0.7, f0, 300, 1, u, nx - 2, 1.0)
    vec["obstacle_in"] = f0
    vec["obstacle_post_stream"] = ps
    vec["obstacle_post_collision"] = pc
    vec["obstacle_meta"] = np.array([nx, ny, 300, 0.52, 0.7, u])
    f_tg = np.empty(16 * 16 * 9)
    O.load_ref(9).ref9_init_taylor_green(16, 2 / 16, 0.62, 1, 1, f_tg)
    vec["tg16_init"] = f_tg
    ps, pc, e = O.ref_run(9, 16, 16, 1, None, 4, 0.62, 0.65, f_tg, 40)
    vec["tg16_erlbm_40_post_collision"] = pc
    ps, pc, e = O.ref_run(9, 16, 16, 1, None, 2, 0.62, 0.62, f_tg, 40)
    vec["tg16_mrt_40_post_collision"] = pc
    f_dsl = np.empty(32 * 32 * 9)
    O.load_ref(9).ref9_init_double_shear(32, 1.0, f_dsl)
    vec["dsl32_init"] = f_dsl
    # the reference's field writers on two stored states: the bytes of every file they write
    import tempfile
    cwd = os.getcwd()
    tmp = tempfile.mkdtemp()
    states = ((9, 16, 16, None, vec["tg16_erlbm_40_post_collision"], "tg16"),
              (19, nx, ny, solid, vec["obstacle_post_collision"], "obstacle"))
    names = {1: "vel_0.500000.vtk", 2: "vor_7.vtk", 3: "rho_7.vtk"}
    for q, a, b, s, f, tag in states:
        sp = None if s is None else np.ascontiguousarray(s, dtype=np.uint8).ctypes.data
        for kind in (1, 2, 3):
            for fmt in (0, 1, 2):
                os.chdir(tmp)
                try:
                    getattr(O.load_ref(q), f"ref{q}_rec_field")(a, b, 1, sp, np.ascontiguousarray(f), kind, fmt,
                                                                 0.5, 7)
                    data = open(names[kind], "rb").read()
                finally:
                    os.chdir(cwd)
                vec[f"vtk_{tag}_field{kind}_format{fmt}"] = np.frombuffer(data, dtype=np.uint8)
    # tools/error_calculator on the ASCII velocity files of two double-shear-layer runs: L = 16 E-RLBM
    # (20 steps) against L = 32 RLBM (40 steps); its erro_L2.dat line carries 10 significant digits
    paths = []
    for L, op, tnh, steps in ((16, 4, 0.65, 20), (32, 3, 1.0, 40)):
        fi = np.empty(L * L * 9)
        O.load_ref(9).ref9_init_double_shear(L, 1.0, fi)
        _, pc, _ = O.ref_run(9, L, L, 1, None, op, 0.5 + 3 * (1 / 32) * L / 80000, tnh, fi, steps)
        os.chdir(tmp)
        try:
            O.load_ref(9).ref9_rec_field(L, L, 1, None, pc, 1, 0, 1.0, 0)
            os.replace("vel_1.000000.vtk", f"vel_L{L}.vtk")
        finally:
            os.chdir(cwd)
        paths.append(f"vel_L{L}.vtk")
    subprocess.run([os.path.join(ROOT, "oracle", "_ref", "error_calculator")] + paths, cwd=tmp, check=True,
                   capture_output=True)
    line = open(os.path.join(tmp, "erro_L2.dat")).read().split()
    vec["errcalc_dsl16_vs_dsl32"] = np.array([16, 32, 20, 40, float(line[1]), float(line[2])])
    # channel boundaries of the library (run_bc): walls at x = 0, nx - 1 and y = 0, ny - 1 (or only
    # y = ny - 1), 25 steps of E-RLBM from a perturbed flow; meta = q nx ny nz walls_y tau tau_nh op
    # steps inlet_x inlet_kind L u_in outlet_x outlet_kind rho_out open_y
    brng = np.random.default_rng(20261204)
    for k, (q, nx_, ny_, nz_, wy, bc) in enumerate(BC_CASES):
        s = channel_mask(nx_, ny_, nz_, wy)
        n_fl = int((s == 0).sum())
        fs = []
        for _ in range(n_fl):
            u = brng.normal(0, 0.03, 3)
            if q == 9:
                u[2] = 0.0
            fs.append(O.equilibrium(q, u[0] + 0.05, u[1], u[2], 1 + brng.normal(0, 0.01)))
        f0 = np.concatenate(fs)
        f0 = f0 + brng.normal(0, 1e-4, f0.size)
        bci = np.array([bc.get("inlet_x", -1), bc.get("inlet_kind", 0), bc.get("parabolic_L", 0),
                        bc.get("outlet_x", -1), bc.get("outlet_kind", 0), bc.get("open_y", -1)], np.int32)
        bcd = np.array([bc.get("u_in", 0.0), bc.get("rho_out", 1.0)])
        ps, pc = np.empty_like(f0), np.empty_like(f0)
        fn = getattr(O.load_ref(q), f"ref{q}_run_bc")
        fn(nx_, ny_, nz_, s.ctypes.data, 4, 0.56, 0.7, f0.ctypes.data, 25, bci.ctypes.data, bcd.ctypes.data,
           ps.ctypes.data, pc.ctypes.data)
        vec[f"bc{k}_in"] = f0
        vec[f"bc{k}_post_collision"] = pc
        vec[f"bc{k}_post_stream_sha256"] = np.frombuffer(hashlib.sha256(ps.tobytes()).digest(), dtype=np.uint8)
        vec[f"bc{k}_meta"] = np.array([q, nx_, ny_, nz_, int(wy), 0.56, 0.7, 4, 25, bci[0], bci[1], bci[2], bcd[0],
                                       bci[3], bci[4], bcd[1], bci[5]], dtype=np.float64)
    # read_geo on a generated geometry file (the file's text is stored too)
    grng = np.random.default_rng(7)
    gx, gy, gz = 9, 5, 2
    vals = (grng.random(gx * gy * gz) > 0.3).astype(int)
    text = ("# vtk DataFile Version 2.0\nGeometria\nASCII\nDATASET STRUCTURED_POINTS\n"
            f"DIMENSIONS {gx} {gy} {gz}\nASPECT_RATIO 1 1 1\nORIGIN 0 0 0\nPOINT_DATA {gx * gy * gz}\n"
            "SCALARS geometria int\nLOOKUP_TABLE default\n" + " ".join(str(v) for v in vals) + "\n")
    gpath = os.path.join(tmp, "geo.vtk")
    with open(gpath, "w") as fgeo:
        fgeo.write(text)
    vec["geo_file"] = np.frombuffer(text.encode(), dtype=np.uint8)
    for pin, pout, wall in ((0, 0, 1), (2, 3, 1), (2, 3, 0)):
        meio = np.zeros((gx + pin + pout) * gy * gz, np.int32)
        lib = O.load_ref(9)
        lib.ref9_read_geo.restype = C.c_int
        nfl = lib.ref9_read_geo(gpath.encode(), pin, pout, wall, meio.ctypes.data_as(C.POINTER(C.c_int)))
        vec[f"geo_ini_{pin}_{pout}_{wall}"] = meio
        vec[f"geo_fluid_{pin}_{pout}_{wall}"] = np.array([nfl])
    np.savez_compressed(os.path.join(HERE, "reference_vectors.npz"), **vec)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
