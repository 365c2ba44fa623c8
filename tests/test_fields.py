"""Field output on the device: the reference's velocity / vorticity / density fields, its VTK writers
(ASCII and big-endian binary, LBM_functions.cpp:4218-5241) and tools/error_calculator.cpp.

FP64: the fields equal the oracle's bit for bit, and the files equal, byte for byte, those the
reference's own writers produced for the same populations (tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_vectors.npz")


def E():
    import erlbm_gb300 as m
    return m


def dsl_lattice(m, L, op, tnh, steps, precision):
    lat = m.Lattice(9, L, L, 1, None, 0.5 + 3 * (1 / 32) * L / 80000, tnh, op, precision)
    lat.set_populations(m.init_double_shear(L))
    lat.step(steps)
    return lat


@pytest.mark.parametrize("case", ["dsl", "obstacle"])
def test_fields_fp64_equal_oracle(case):
    m = E()
    if case == "dsl":
        L = 64
        lat = dsl_lattice(m, L, m.OP_EXTREG, 0.65, 25, m.FP64)
        q, nx, ny, solid = 9, L, L, None
    else:
        nx, ny, solid = O.obstacle_geometry()
        q = 19
        lat = m.Lattice(19, nx, ny, 1, solid, 0.52, 0.7, m.OP_EXTREG, m.FP64)
        lat.set_populations(np.tile(O.equilibrium(19, 0, 0, 0, 1.0), lat.n_fluid))
        lat.step(200, dict(inlet_x=1, u_in=0.05, outlet_x=nx - 2, rho_out=1.0))
    with lat:
        for stage in (m.STAGE_POST_STREAM, m.STAGE_POST_COLLISION):
            f = lat.get_populations(stage)
            for kind in (m.FIELD_VELOCITY, m.FIELD_VORTICITY, m.FIELD_DENSITY):
                got = lat.field(kind, stage).reshape(-1)
                assert np.array_equal(got, O.field(q, nx, ny, 1, solid, f, kind)), (stage, kind)


@pytest.mark.parametrize("tag", ["tg16", "obstacle"])
def test_vtk_files_equal_reference_writers(tag, tmp_path):
    m = E()
    v = np.load(GOLD)
    if tag == "tg16":
        q, nx, ny, solid, f = 9, 16, 16, None, v["tg16_erlbm_40_post_collision"]
    else:
        nx, ny, solid = O.obstacle_geometry()
        q, f = 19, v["obstacle_post_collision"]
    with m.Lattice(q, nx, ny, 1, solid, 0.6, 0.65, m.OP_EXTREG, m.FP64) as lat:
        lat.set_populations(f)  # the given populations are the post-stream stage until a step runs
        for kind in (1, 2, 3):
            for fmt in (0, 1, 2):
                path = tmp_path / f"{kind}_{fmt}.vtk"
                lat.write_vtk(str(path), kind, fmt, m.STAGE_POST_STREAM)
                assert path.read_bytes() == v[f"vtk_{tag}_field{kind}_format{fmt}"].tobytes(), (kind, fmt)


def test_vtk_large_lattice_matches_oracle(tmp_path):
    """L = 512: the threaded ASCII formatting and the device big-endian encoding against the oracle."""
    m = E()
    L = 512
    with dsl_lattice(m, L, m.OP_REG, 1.0, 10, m.FP64) as lat:
        f = lat.get_populations(m.STAGE_POST_COLLISION)
        for kind, fmt in ((1, 0), (2, 1), (3, 2), (1, 2)):
            a, b = tmp_path / "gpu.vtk", tmp_path / "orc.vtk"
            lat.write_vtk(str(a), kind, fmt)
            O.write_vtk(9, L, L, 1, None, f, kind, fmt, str(b))
            assert a.read_bytes() == b.read_bytes(), (kind, fmt)


def test_error_calculator_equals_tool():
    """The device run of the error pipeline (FP64 lattices, 6-digit text rounding) gives the values
    tools/error_calculator printed for the reference's files, to its 10 digits; full precision agrees
    with the oracle's full-precision errors to 1e-12."""
    m = E()
    v = np.load(GOLD)
    Ls, Lr, ns, nr, ev, em = v["errcalc_dsl16_vs_dsl32"]
    with dsl_lattice(m, int(Ls), m.OP_EXTREG, 0.65, int(ns), m.FP64) as sim, \
            dsl_lattice(m, int(Lr), m.OP_REG, 1.0, int(nr), m.FP64) as ref:
        e6 = m.velocity_error(sim, ref, text_digits=6)
        assert float(f"{e6[0]:.10g}") == ev and float(f"{e6[1]:.10g}") == em
        e0 = m.velocity_error(sim, ref)
        vs = O.field(9, int(Ls), int(Ls), 1, None, sim.get_populations(1), 1)
        vr = O.field(9, int(Lr), int(Lr), 1, None, ref.get_populations(1), 1)
        want = O.velocity_error(int(Ls), int(Ls), vs, int(Lr), int(Lr), vr)
        np.testing.assert_allclose(e0, want, rtol=1e-12)
        assert O.velocity_error(int(Ls), int(Ls), vs, int(Lr), int(Lr), vr, 6) == e6


def test_fp32_fields_close_to_fp64():
    m = E()
    L = 256
    with dsl_lattice(m, L, m.OP_EXTREG, 0.65, 50, m.FP64) as a, dsl_lattice(m, L, m.OP_EXTREG, 0.65, 50,
                                                                             m.FP32_SHIFTED) as b:
        # relative errors of u, of the vorticity and of rho - 1 (FP32-shifted stores g = f - w)
        for kind, tol, shift in ((m.FIELD_VELOCITY, 1e-5, 0.0), (m.FIELD_VORTICITY, 1e-4, 0.0),
                                 (m.FIELD_DENSITY, 1e-4, 1.0)):
            x, y = a.field(kind), b.field(kind)
            assert np.linalg.norm(y - x) / np.linalg.norm(x - shift) < tol, kind
        e = m.velocity_error(b, a)
        assert e[0] < 1e-5


def test_field_argument_checks():
    m = E()
    with m.Lattice(9, 8, 8, 1, None, 0.6, 0.65, m.OP_EXTREG, m.FP64) as a, \
            m.Lattice(9, 12, 12, 1, None, 0.6, 0.65, m.OP_EXTREG, m.FP64) as b:
        a.set_populations(np.tile(O.equilibrium(9, 0, 0, 0, 1.0), 64))
        b.set_populations(np.tile(O.equilibrium(9, 0, 0, 0, 1.0), 144))
        with pytest.raises(m.ErlbmError) as ei:
            m.velocity_error(a, b, sim_stage=0, ref_stage=0)  # 12 is not a multiple of 8
        assert ei.value.code == -1
        with pytest.raises(m.ErlbmError) as ei:
            a.field(m.FIELD_VELOCITY, m.STAGE_POST_COLLISION)  # no collision has run yet
        assert ei.value.code == -7


def test_fig4_rows_reproduced_at_full_size():
    """The published Fig. 4 table (data/fig4_double_shear_Re80000.csv) comes from an RLBM run at
    L = 2048 and the error tool on 6-digit ASCII files.  The FP64 pipeline on the GPU -- the L = 2048
    reference (65 537 steps) and the L = 64 runs of all three models -- gives the published E_vector
    and E_magnitude to their 6 printed digits.  (About 80 s on a GB300.)"""
    import json
    from erlbm_gb300 import programs as P
    m = E()
    with open(os.path.join(os.path.dirname(GOLD), "published.json")) as f:
        pub = json.load(f)["fig4_double_shear_Re80000"]
    rows = P.fig4_table(Ls=(64,), precision=m.FP64)
    assert len(rows) == 3
    for r in rows:
        p = next(x for x in pub if x["model"] == r["model"] and int(x["L"]) == r["L"])
        assert float(f"{r['E_vector']:.6g}") == p["E_vector"] and float(f"{r['E_magnitude']:.6g}") == p["E_magnitude"]
