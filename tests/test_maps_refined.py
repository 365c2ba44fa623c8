"""FP32-screened stability maps with FP64 refinement of the boundary points (erlbm_map_run_refined).

The refined map must hold, at every refined point, exactly the FP64 map's result (the reference's
labels, decided steps and margins), at every other point exactly the FP32-shifted map's result, and
its selection must be the documented rule applied to the FP32 labels.  Small grids with capped run
budgets keep each map to seconds.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def E():
    import erlbm_gb300 as m
    return m


def selection(lab32, dec32, budgets, n_i, n_j, radius, late):
    """The refinement rule restated in numpy on one operator plane."""
    L = lab32.reshape(n_j, n_i)
    P = np.pad(L, radius, mode="edge")
    hi, lo = L.copy(), L.copy()
    for dj in range(-radius, radius + 1):
        for di in range(-radius, radius + 1):
            S = P[radius + dj:radius + dj + n_j, radius + di:radius + di + n_i]
            hi, lo = np.maximum(hi, S), np.minimum(lo, S)
    sel = (hi != lo).reshape(-1)
    if late > 0:
        sel |= (lab32 == 1) & (dec32 > late * budgets)
    return sel


def budgets(kind, n_i, n_j, op, cap):
    m = E()
    out = []
    for j in range(n_j):
        for i in range(n_i):
            if kind == m.MAP_TAYLOR_GREEN:
                u0 = m.tg_map_params(i, j, n_i, n_j, op, 0.65)[0]
                n = int(1600.0 / u0)
            else:
                nx, ny, _ = m.obstacle_geometry()
                n = int(200.0 * ny / m.obstacle_map_params(i, j, n_i, n_j)[0])
            out.append(min(n, cap))
    return np.array(out, np.float64)


@pytest.mark.parametrize("kind,n,cap", [(1, 24, 4000), (2, 20, 3000)])
def test_refined_map_takes_fp64_results_where_it_refines(kind, n, cap):
    m = E()
    op = 0 if kind == m.MAP_TAYLOR_GREEN else m.OP_EXTREG
    radius, late = 1, 0.3
    lab, dec, mg, ref = m.map_run_refined(kind, op=op, n_i=n, n_j=n, max_steps=cap, radius=radius,
                                          late_fraction=late)
    l64, d64, m64 = m.map_run(kind, None, precision=m.FP64, op=op, n_i=n, n_j=n, max_steps=cap)
    l32, d32, m32 = m.map_run(kind, None, precision=m.FP32_SHIFTED, op=op, n_i=n, n_j=n, max_steps=cap)
    assert ref.any()
    np.testing.assert_array_equal(lab[ref], l64[ref])
    np.testing.assert_array_equal(dec[ref], d64[ref])
    np.testing.assert_array_equal(mg[ref], m64[ref])
    np.testing.assert_array_equal(lab[~ref], l32[~ref])
    np.testing.assert_array_equal(dec[~ref], d32[~ref])
    np.testing.assert_array_equal(mg[~ref], m32[~ref])
    ops = [m.OP_REG, m.OP_EXTREG] if op == 0 else [op]
    planes = n * n
    for o, opk in enumerate(ops):
        sl = slice(o * planes, (o + 1) * planes)
        want = selection(l32[sl], d32[sl], budgets(kind, n, n, opk, cap), n, n, radius, late)
        np.testing.assert_array_equal(ref[sl], want)
    assert np.mean(lab == l64) >= np.mean(l32 == l64)

