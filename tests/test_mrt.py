"""coll_MRT (Collision_operators.cpp:487-701; a D2Q9-only operator in the reference,
src/erlbm_common.h:74-76) on every path that takes an operator: the single lattice in FP64
(bit-identical to the oracle and to the reference's own golden vectors) and in FP32-shifted (error
bounds stated below), the fused periodic kernel, batched runs and the request server."""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_vectors.npz")


def E():
    import erlbm_gb300 as m
    return m


def random_state(n, rng, amp=0.05, noise=1e-3):
    fs = [O.equilibrium(9, *rng.normal(0, amp, 2), 0.0, 1 + rng.normal(0, 0.01)) for _ in range(n)]
    f = np.concatenate(fs)
    return f + rng.normal(0, noise, f.size)


@pytest.mark.parametrize("nx,ny", [(7, 5), (32, 32), (256, 8)])
def test_mrt_fp64_bitwise(nx, ny):
    m = E()
    rng = np.random.default_rng(nx * ny)
    ref = O.Lattice(9, nx, ny, 1, None, 0.57, 0.57, O.OP_MRT)
    f0 = random_state(ref.n_fluid, rng)
    ref.set(f0)
    ref.step(13)
    with m.Lattice(9, nx, ny, 1, None, 0.57, 0.57, m.OP_MRT, m.FP64) as lat:
        lat.set_populations(f0)
        lat.step(13)
        assert np.array_equal(lat.get_populations(m.STAGE_POST_STREAM), ref.get(0))
        assert np.array_equal(lat.get_populations(m.STAGE_POST_COLLISION), ref.get(1))
        assert lat.kinetic_energy(0) == ref.kinetic_energy(0)


def test_mrt_fp64_reference_vectors():
    """Against runs of the reference library itself (tests/golden/make_golden.py)."""
    m = E()
    v = np.load(GOLD)
    nx, ny, nz, steps, _, tau, tnh = v["periodic_q9_op2_meta"]
    with m.Lattice(9, int(nx), int(ny), 1, None, tau, tnh, m.OP_MRT, m.FP64) as lat:
        lat.set_populations(v["periodic_q9_op2_in"])
        lat.step(int(steps))
        assert np.array_equal(lat.get_populations(0), v["periodic_q9_op2_post_stream"])
        assert np.array_equal(lat.get_populations(1), v["periodic_q9_op2_post_collision"])
        assert lat.kinetic_energy(0) == float(v["periodic_q9_op2_energy"][0])
    with m.Lattice(9, 16, 16, 1, None, 0.62, 0.62, m.OP_MRT, m.FP64) as lat:
        lat.set_populations(v["tg16_init"])
        lat.step(40)
        assert np.array_equal(lat.get_populations(1), v["tg16_mrt_40_post_collision"])


def test_mrt_fp32_shifted_close():
    """Relative error of the shifted populations g = f - w after 50 steps: < 2e-6."""
    m = E()
    rng = np.random.default_rng(11)
    nx, ny, tau = 40, 24, 0.6
    ref = O.Lattice(9, nx, ny, 1, None, tau, tau, O.OP_MRT)
    f0 = random_state(ref.n_fluid, rng, amp=0.03, noise=1e-4)
    ref.set(f0)
    ref.step(50)
    with m.Lattice(9, nx, ny, 1, None, tau, tau, m.OP_MRT, m.FP32_SHIFTED) as lat:
        lat.set_populations(f0)
        lat.step(50)
        f = lat.get_populations(0)
    w = np.tile(O.equilibrium(9, 0, 0, 0, 1.0), ref.n_fluid)
    rel = np.linalg.norm((f - w) - (ref.get(0) - w)) / np.linalg.norm(ref.get(0) - w)
    assert rel < 2e-6, rel


def test_mrt_fused_periodic_kernel():
    """The fused D2Q9 kernel (nx % 128 == 0) on the double shear layer at its Re = 80000 viscosity:
    relative error of g after 20 steps < 1e-5, and mass conserved to FP32 rounding."""
    m = E()
    L = 256
    tau = 0.5 + 3 * (1 / 32) * L / 80000
    f0 = m.init_double_shear(L)
    ref = O.Lattice(9, L, L, 1, None, tau, tau, O.OP_MRT)
    ref.set(f0)
    ref.step(20)
    with m.Lattice(9, L, L, 1, None, tau, tau, m.OP_MRT, m.FP32_SHIFTED) as lat:
        lat.set_populations(f0)
        lat.step(20)
        f = lat.get_populations(1)
    w = np.tile(O.equilibrium(9, 0, 0, 0, 1.0), L * L)
    rel = np.linalg.norm(f - ref.get(1)) / np.linalg.norm(ref.get(1) - w)
    assert rel < 1e-5, rel
    assert abs(f.sum() - f0.sum()) < 1e-6 * L * L


def test_mrt_batched_and_served_runs():
    """Batched D2Q9 runs and a served Taylor-Green request under MRT equal single-lattice oracle runs."""
    m = E()
    rng = np.random.default_rng(5)
    L = 12
    runs, blocks = [], []
    for k in range(4):
        u0 = 0.02 + 0.01 * k
        f0 = O.init_taylor_green(9, L, u0, 0.6) + rng.normal(0, 1e-5, L * L * 9)
        blocks.append(f0)
        runs.append(dict(op=m.OP_MRT, tau=0.55 + 0.02 * k, tau_nh=1.0, u0=u0, n_steps=40 + 30 * k,
                         aos_offset=k * f0.size))
    res = m.batch_run(9, L, L, runs, precision=m.FP64, init=m.INIT_AOS, aos=np.concatenate(blocks),
                      energy_every=10, energy_factor=2.0)
    for k, r in enumerate(runs):
        last = (r["n_steps"] - 1) // 10 * 10
        lat = O.Lattice(9, L, L, 1, None, r["tau"], r["tau"], O.OP_MRT)
        lat.set(blocks[k])
        lat.step(last)
        assert res[k]["label"] == 0 and res[k]["steps_done"] == r["n_steps"]
        assert res[k]["energy"] == lat.kinetic_energy(0)
    with m.Server(hbm_budget_bytes=1 << 28) as srv:
        L, u0 = 32, 2 / 32
        tau = 0.5 + 3 * u0 * L / 50
        r = srv.wait(srv.submit(m.REQ_TG2D, m.FP64, op=m.OP_MRT, L=L, tau=tau, tau_nh=tau, u0=u0, n_steps=61))
        lat = O.Lattice(9, L, L, 1, None, tau, tau, O.OP_MRT)
        lat.set(O.init_taylor_green(9, L, u0, tau))
        lat.step(61)
        assert r["status"] == 0 and r["energy"] == lat.kinetic_energy(0)


def test_mrt_is_d2q9_only():
    m = E()
    with pytest.raises(m.ErlbmError) as ei:
        m.batch_run(19, 16, 16, [dict(op=m.OP_MRT, tau=0.6, tau_nh=0.6, u0=0.01, n_steps=10)],
                    init=m.INIT_TG_MAP)
    assert ei.value.code == -6
    with m.Lattice(19, 4, 4, 1, None, 0.6, 0.6, m.OP_EXTREG, m.FP64) as lat:
        with pytest.raises(m.ErlbmError) as ei:
            lat.set_params(0.6, 0.6, m.OP_MRT)
        assert ei.value.code == -6
