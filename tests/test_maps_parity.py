"""GPU parity of the batched stability-map path against the CPU oracle.

FP64: labels, decided steps and margins identical to the oracle's roda_ponto restatement.
FP32-shifted: label agreement with FP64 reported and bounded.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def eg():
    import erlbm_gb300 as E
    return E


# a spread of map points: corners, middle and the unstable region (i = U0 axis, j = viscosity axis)
TG_POINTS = [(399, 0), (300, 20), (200, 100), (10, 300), (0, 399), (50, 50), (120, 10), (399, 399), (5, 0),
             (60, 180), (250, 250), (30, 390)]
OB_POINTS = [(0, 0), (200, 200), (399, 399), (10, 5), (100, 40), (300, 10), (50, 300), (390, 100)]


@pytest.mark.parametrize("op", [3, 4])
def test_tg_map_fp64_matches_oracle(op):
    cap = 3000
    lab, dec, mg = eg().map_run(eg().MAP_TAYLOR_GREEN, TG_POINTS, precision=eg().FP64, op=op, tau_nh=0.65,
                                max_steps=cap)
    olab, odec, omg = O.tg_map(TG_POINTS, op=op, tau_nh=0.65, max_steps=cap)
    assert np.array_equal(lab, olab)
    assert np.array_equal(dec, odec)
    assert np.array_equal(mg, omg)


def test_tg_map_both_ops_one_launch():
    cap = 2000
    lab, dec, mg = eg().map_run(eg().MAP_TAYLOR_GREEN, TG_POINTS, precision=eg().FP64, op=0, max_steps=cap)
    n = len(TG_POINTS)
    for k, op in enumerate((3, 4)):
        olab, odec, _ = O.tg_map(TG_POINTS, op=op, tau_nh=0.65, max_steps=cap)
        assert np.array_equal(lab[k * n:(k + 1) * n], olab)
        assert np.array_equal(dec[k * n:(k + 1) * n], odec)


def test_obstacle_map_fp64_matches_oracle():
    cap = 2500
    lab, dec, mg = eg().map_run(eg().MAP_OBSTACLE, OB_POINTS, precision=eg().FP64, max_steps=cap)
    olab, odec, omg = O.obstacle_map(OB_POINTS, max_steps=cap)
    assert np.array_equal(lab, olab)
    assert np.array_equal(dec, odec)
    assert np.array_equal(mg, omg)


def test_maps_fp32_label_agreement():
    """FP32-shifted vs FP64 labels; disagreements sit at the stability boundary (see DESIGN)."""
    pts = [(i, j) for i in range(0, 400, 40) for j in range(0, 400, 40)]
    cap = 3000
    for kind in (eg().MAP_TAYLOR_GREEN, eg().MAP_OBSTACLE):
        l64, d64, m64 = eg().map_run(kind, pts, precision=eg().FP64, op=4, max_steps=cap)
        l32, d32, m32 = eg().map_run(kind, pts, precision=eg().FP32_SHIFTED, op=4, max_steps=cap)
        agree = np.mean(l64 == l32)
        assert agree >= 0.9, (kind, agree)
        # runs that both precisions call stable agree on the margin to ~1e-4 (same physics)
        both = (l64 == 0) & (l32 == 0)
        assert np.all(np.abs(m32[both] - m64[both]) <= 1e-3 * np.abs(m64[both]) + 1e-6)


def test_batch_run_aos_init_matches_lattice_runs():
    """erlbm_batch_run with per-run initial populations equals single-lattice oracle runs."""
    rng = np.random.default_rng(3)
    L = 12
    runs, blocks = [], []
    for k in range(6):
        u0 = 0.02 + 0.01 * k
        f0 = O.init_taylor_green(9, L, u0, 0.6)
        f0 = f0 + rng.normal(0, 1e-5, f0.size)
        blocks.append(f0)
        runs.append(dict(op=[1, 3, 4][k % 3], tau=0.55 + 0.02 * k, tau_nh=0.7, u0=u0, n_steps=50 + 37 * k,
                         aos_offset=k * f0.size))
    aos = np.concatenate(blocks)
    res = eg().batch_run(9, L, L, runs, precision=eg().FP64, init=eg().INIT_AOS, aos=aos, energy_every=10,
                         energy_factor=2.0)
    for k, r in enumerate(runs):
        lat = O.Lattice(9, L, L, 1, None, r["tau"], r["tau_nh"], r["op"])
        lat.set(blocks[k])
        e0 = lat.kinetic_energy(0)
        lat.step(r["n_steps"])
        assert res[k]["label"] == 0 and res[k]["steps_done"] == r["n_steps"]
        # the last energy check ran at the last multiple of 10 below n_steps: compare E there
        last = (r["n_steps"] - 1) // 10 * 10
        lat2 = O.Lattice(9, L, L, 1, None, r["tau"], r["tau_nh"], r["op"])
        lat2.set(blocks[k])
        lat2.step(last)
        assert res[k]["energy"] == (lat2.kinetic_energy(0) if last > 0 else e0)


def test_sharded_map_world1_equals_map_run():
    """map_run_sharded, the multi-GPU map of bench.py, in a one-rank run: the same labels, decided
    steps and margins as map_run on the same points, both operators of the Taylor-Green map."""
    import erlbm_gb300 as m
    from erlbm_gb300.sharding import map_run_sharded
    pts = [(i, j) for i in range(0, 400, 53) for j in range(0, 400, 67)]
    for kind, op in ((m.MAP_TAYLOR_GREEN, 0), (m.MAP_OBSTACLE, m.OP_EXTREG)):
        a = m.map_run(kind, pts, precision=m.FP64, op=op, max_steps=1200)
        b = map_run_sharded(kind, pts, precision=m.FP64, op=op, max_steps=1200)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def fp32_cta_shape(nb):
    """The FP32 batched kernel's CTA for an nb-node lattice (two nodes per thread, whole warps)."""
    return ((nb + 1) // 2 + 31) // 32 * 32, 2


def same_result(gpu, cpu):
    for k in ("label", "decided_step", "steps_done", "status", "margin", "energy"):
        a, b = gpu[k], cpu[k]
        if not (a == b or (a != a and b != b)):
            return False
    return True


def test_fp32_map_kernel_equals_its_cpu_restatement():
    """The FP32-shifted batched map kernel (k_batch over PrecShifted32) against its CPU restatement
    (oracle/fp32_shifted.c, orc32_batch_run): label, decided step, steps done, status, margin and energy
    bit for bit, on 40 Taylor-Green map points (RLBM and E-RLBM, energy checks every 100 steps, whose
    sum follows the kernel's thread slots and reduction tree) and 24 obstacle points (Zou-He inlet,
    density outlet, bounce-back, FP32 density check every step), each run to a capped budget.  The runs
    are roda_ponto of main_stability-map_taylor-green.cpp:41-104 and main_stability-map_obstacle.cpp:75-123."""
    import erlbm_gb300 as m
    runs = []
    for k in range(40):
        op = m.OP_EXTREG if k % 2 else m.OP_REG
        u0, tau, tnh = m.tg_map_params((31 * k + 7) % 400, (83 * k + 11) % 400, 400, 400, op, 0.65)
        runs.append(dict(op=op, tau=tau, tau_nh=tnh, u0=u0, n_steps=4000))
    got = m.batch_run(19, 16, 16, runs, precision=m.FP32_SHIFTED, energy_every=100, energy_factor=2.0,
                      init=m.INIT_TG_MAP)
    block, npt = fp32_cta_shape(256)
    unstable = 0
    for r, g in zip(runs, got):
        want = O.fp32_batch_run(19, 16, 16, r["op"], r["tau"], r["tau_nh"], r["u0"], r["n_steps"], block, npt,
                                energy_every=100, energy_factor=2.0, init=1)
        assert same_result(g, want), (r, g, want)
        unstable += g["label"]
    assert 0 < unstable < len(runs)
    nx, ny, solid = m.obstacle_geometry()
    runs = []
    for k in range(24):
        u, tau, tnh = m.obstacle_map_params((53 * k + 3) % 400, (29 * k + 7) % 400)
        runs.append(dict(op=m.OP_EXTREG, tau=tau, tau_nh=tnh, u0=u, n_steps=3000))
    got = m.batch_run(19, nx, ny, runs, precision=m.FP32_SHIFTED, solid=solid, inlet_x=1, outlet_x=nx - 2,
                      density_check=True, density_limit=10.0, init=m.INIT_REST)
    block, npt = fp32_cta_shape(nx * ny)
    unstable = 0
    for r, g in zip(runs, got):
        want = O.fp32_batch_run(19, nx, ny, r["op"], r["tau"], r["tau_nh"], r["u0"], r["n_steps"], block, npt,
                                solid=solid, inlet_x=1, outlet_x=nx - 2, density_check=True, density_limit=10.0,
                                init=0)
        assert same_result(g, want), (r, g, want)
        unstable += g["label"]
    assert 0 < unstable < len(runs)
