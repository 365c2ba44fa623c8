"""The library's channel boundaries on the GPU (Boundary_conditions.cpp): Zou-He D2Q9 and parabolic
inlets, open and convective outlets, the open y plane, next to devnull_rho_x and the D3Q19 Zou-He inlet.

FP64: bit-identical to runs of the reference library (tests/golden) and to the oracle over a longer
run on a geometry read with read_geo.  FP32-shifted: relative error bound stated per test.
"""
import hashlib
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_vectors.npz")


def E():
    import erlbm_gb300 as m
    return m


def channel_mask(nx, ny, nz, walls_y):
    s = np.zeros((nz, ny, nx), np.uint8)
    s[:, :, 0] = 1
    s[:, :, nx - 1] = 1
    s[:, ny - 1, :] = 1
    if walls_y:
        s[:, 0, :] = 1
    return s.reshape(-1)


def case(v, k):
    mt = v[f"bc{k}_meta"]
    q, nx, ny, nz, wy = (int(x) for x in mt[:5])
    bc = dict(inlet_x=int(mt[9]), inlet_kind=int(mt[10]), parabolic_L=int(mt[11]), u_in=mt[12],
              outlet_x=int(mt[13]), outlet_kind=int(mt[14]), rho_out=mt[15], open_y=int(mt[16]))
    return q, nx, ny, nz, channel_mask(nx, ny, nz, bool(wy)), mt[5], mt[6], int(mt[7]), int(mt[8]), bc


@pytest.mark.parametrize("k", range(6))
def test_channel_boundaries_fp64_equal_reference(k):
    m = E()
    v = np.load(GOLD)
    q, nx, ny, nz, solid, tau, tnh, op, steps, bc = case(v, k)
    with m.Lattice(q, nx, ny, nz, solid, tau, tnh, op, m.FP64) as lat:
        lat.set_populations(v[f"bc{k}_in"])
        lat.step(steps, bc)
        assert np.array_equal(lat.get_populations(m.STAGE_POST_COLLISION), v[f"bc{k}_post_collision"])
        ps = lat.get_populations(m.STAGE_POST_STREAM)
        assert hashlib.sha256(ps.tobytes()).digest() == v[f"bc{k}_post_stream_sha256"].tobytes()


@pytest.mark.parametrize("k", range(6))
def test_channel_boundaries_fp32_close(k):
    """FP32-shifted against the oracle after the same 25 steps: relative error of g = f - w < 1e-5."""
    m = E()
    v = np.load(GOLD)
    q, nx, ny, nz, solid, tau, tnh, op, steps, bc = case(v, k)
    with m.Lattice(q, nx, ny, nz, solid, tau, tnh, op, m.FP32_SHIFTED) as lat:
        lat.set_populations(v[f"bc{k}_in"])
        lat.step(steps, bc)
        f = lat.get_populations(m.STAGE_POST_COLLISION)
    ref = v[f"bc{k}_post_collision"]
    w = np.tile(O.equilibrium(q, 0, 0, 0, 1.0), ref.size // q)
    rel = np.linalg.norm(f - ref) / np.linalg.norm(ref - w)
    assert rel < 1e-5, rel


def test_channel_from_read_geo_long_run(tmp_path):
    """A channel with an obstacle written as a geometry file, read with read_geo (inlet and outlet
    layers with walls), 600 steps with a parabolic inlet and a convective outlet: FP64 equals the
    oracle bit for bit."""
    m = E()
    gx, gy = 30, 14
    geo = np.ones((gy, gx), int)
    geo[0, :] = 0
    geo[gy - 1, :] = 0
    geo[5:9, 8:11] = 0
    text = ("# vtk DataFile Version 2.0\ncanal\nASCII\nDATASET STRUCTURED_POINTS\n"
            f"DIMENSIONS {gx} {gy} 1\nASPECT_RATIO 1 1 1\nORIGIN 0 0 0\nPOINT_DATA {gx * gy}\n"
            "SCALARS geometria int\nLOOKUP_TABLE default\n" + " ".join(str(x) for x in geo.reshape(-1)) + "\n")
    path = tmp_path / "canal.vtk"
    path.write_text(text)
    nx, ny, nz, solid = m.read_geo(str(path), 2, 2, True)
    assert np.array_equal(solid, O.read_geo(str(path), 2, 2, True)[3])
    for q, op in ((9, m.OP_EXTREG), (9, m.OP_MRT)):
        bc = dict(inlet_x=2, inlet_kind=m.INLET_PARABOLIC, parabolic_L=12, u_in=0.05, outlet_x=nx - 2,
                  outlet_kind=m.OUTLET_CONVECTIVE)
        ref = O.Lattice(q, nx, ny, nz, solid, 0.55, 0.7, op)
        f0 = np.tile(O.equilibrium(q, 0, 0, 0, 1.0), ref.n_fluid)
        ref.set(f0)
        ref.step(600, bc)
        with m.Lattice(q, nx, ny, nz, solid, 0.55, 0.7, op, m.FP64) as lat:
            lat.set_populations(f0)
            lat.step(600, bc)
            assert np.array_equal(lat.get_populations(m.STAGE_POST_COLLISION), ref.get(1))


def test_channel_boundary_checks():
    m = E()
    solid = channel_mask(12, 8, 2, True)
    with m.Lattice(19, 12, 8, 2, solid, 0.6, 0.7, m.OP_EXTREG, m.FP64) as lat:
        lat.set_populations(np.tile(O.equilibrium(19, 0, 0, 0, 1.0), lat.n_fluid))
        with pytest.raises(m.ErlbmError) as ei:  # open outlet: a D2Q9 boundary
            lat.step(1, dict(outlet_x=10, outlet_kind=m.OUTLET_OPEN))
        assert ei.value.code == -6
        with pytest.raises(m.ErlbmError) as ei:  # 6 fluid nodes per column > L = 5
            lat.step(1, dict(inlet_x=1, inlet_kind=m.INLET_PARABOLIC, parabolic_L=5, u_in=0.05))
        assert ei.value.code == -1
        with pytest.raises(m.ErlbmError) as ei:  # L must stay below ny
            lat.step(1, dict(inlet_x=1, inlet_kind=m.INLET_PARABOLIC, parabolic_L=8, u_in=0.05))
        assert ei.value.code == -1
        with pytest.raises(m.ErlbmError) as ei:  # the open y plane is a D2Q9 boundary
            lat.step(1, dict(open_y=1))
        assert ei.value.code == -6
