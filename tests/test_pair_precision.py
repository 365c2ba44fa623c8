"""The compensated FP32 form (ERLBM_FP32_PAIR): populations stored as float pairs and collided in
float-float arithmetic on the FP32 pipe.

CPU: its restatement (oracle/fp32_shifted.c, orc32p_periodic_d2q9) stays within 1e-11 of the FP64
oracle (the reference's results), where the FP32-shifted restatement sits at ~1e-7.
GPU: the kernel reproduces the restatement bit for bit, and on the double shear layer its velocity
error against FP64 at t* = 1 is below the 1e-5 target that FP32 storage misses.
"""
import numpy as np
import pytest

from oracle import oracle as O


def E():
    import erlbm_gb300 as m
    return m


def near_eq(nx, ny, seed, amp=0.05):
    rng = np.random.default_rng(seed)
    w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
    return (w[None, :] * (1.0 + amp * rng.standard_normal((nx * ny, 9)))).ravel()


@pytest.mark.parametrize("op", [1, 3, 4])
def test_pair_restatement_tracks_the_fp64_oracle(op):
    nx, ny, steps = 24, 20, 150
    f0 = near_eq(nx, ny, op)
    tau, tnh = 0.51, 0.65
    pair = O.fp32_pair_periodic_d2q9(nx, ny, op, tau, tnh, f0, steps)
    f32 = O.fp32_periodic_d2q9(nx, ny, op, tau, tnh, f0, steps)
    ref = O.Lattice(9, nx, ny, 1, None, tau, tnh, op)
    ref.set(f0)
    ref.step(steps)
    want = ref.get(1)
    w = np.tile(O.equilibrium(9, 0, 0, 0, 1.0), nx * ny)
    scale = np.linalg.norm(want - w)
    e_pair = np.linalg.norm(pair - want) / scale
    e_f32 = np.linalg.norm(f32 - want) / scale
    assert e_pair < 1e-11, e_pair
    assert e_pair < 1e-3 * e_f32


def test_pair_precision_limits_are_refused():
    m = E()
    for kw in (dict(q=19, nx=8, ny=8, nz=8, op=m.OP_EXTREG), dict(q=9, nx=8, ny=8, nz=1, op=m.OP_MRT)):
        with pytest.raises(m.ErlbmError) as ei:
            m.Lattice(kw["q"], kw["nx"], kw["ny"], kw["nz"], None, 0.6, 0.65, kw["op"], m.FP32_PAIR)
        assert ei.value.code == -6
    solid = np.zeros(64, np.uint8)
    solid[5] = 1
    with pytest.raises(m.ErlbmError) as ei:
        m.Lattice(9, 8, 8, 1, solid, 0.6, 0.65, m.OP_EXTREG, m.FP32_PAIR)
    assert ei.value.code == -6


@pytest.mark.gpu
@pytest.mark.parametrize("op", [1, 3, 4])
def test_pair_kernel_equals_its_cpu_restatement(op):
    """The compensated kernel on a 72 x 40 periodic box (random near-equilibrium populations, the
    first step in place, then pulls) gives the restatement's populations bit for bit."""
    m = E()
    nx, ny, steps = 72, 40, 37
    f0 = near_eq(nx, ny, 10 + op)
    tau, tnh = 0.53, 0.65
    want = O.fp32_pair_periodic_d2q9(nx, ny, op, tau, tnh, f0, steps)
    with m.Lattice(9, nx, ny, 1, None, tau, tnh, op, m.FP32_PAIR) as lat:
        lat.set_populations(f0)
        lat.step(20)
        lat.step(steps - 20)
        got = lat.get_populations(m.STAGE_POST_COLLISION)
    assert np.array_equal(got, want)


@pytest.mark.gpu
def test_pair_meets_the_velocity_error_target_on_the_double_shear_layer():
    """The double shear layer (Re = 80000, E-RLBM tau_nh = 0.65) at L = 512 to t* = 1: the compensated
    form's relative L2 velocity error against FP64 is below the 1e-5 target for the FP32 forms, where
    the FP32-shifted form's is above it."""
    from erlbm_gb300 import programs as P
    pair = P.precision_error(512, t_stars=(0.5, 1.0), precision=E().FP32_PAIR)
    f32 = P.precision_error(512, t_stars=(1.0,), precision=E().FP32_SHIFTED)
    print("pair", pair, "fp32", f32)
    assert pair[1.0] < 1e-5
    assert pair[1.0] < 0.01 * f32[1.0]
