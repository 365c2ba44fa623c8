"""The GPU stability maps against the reference itself: labels of the reference's own roda_ponto
(compiled from its sources; tests/golden/reference_maps_20x20.json) on the README's 20 x 20
subsample, full run lengths.  The plain FP64 path must reproduce every label."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def ref():
    with open(os.path.join(GOLD, "reference_maps_20x20.json")) as f:
        return json.load(f)


def E():
    import erlbm_gb300 as m
    return m


def test_tg_map_fp64_equals_reference_labels():
    m = ref()
    pts = [tuple(p) for p in m["tg_points"]]
    lab, dec, mg = E().map_run(E().MAP_TAYLOR_GREEN, pts, precision=E().FP64, op=0, tau_nh=0.65)
    assert list(lab[:400]) == m["tg_reg"]
    assert list(lab[400:]) == m["tg_erlbm065"]


def test_obstacle_map_fp64_equals_reference_labels():
    m = ref()
    pts = [tuple(p) for p in m["obstacle_points"]]
    lab, dec, mg = E().map_run(E().MAP_OBSTACLE, pts, precision=E().FP64)
    assert list(lab) == m["obstacle"]


def test_20x20_runs_fp64_equal_reference_labels():
    """The README's quick-test protocol: whole 20 x 20 maps (axes computed with n = 20)."""
    m = ref()
    if "grid20_tg_reg" not in m:
        pytest.skip("fixture without the 20 x 20 runs")
    lab, _, _ = E().map_run(E().MAP_TAYLOR_GREEN, None, precision=E().FP64, op=0, tau_nh=0.65, n_i=20, n_j=20)
    assert list(lab[:400]) == m["grid20_tg_reg"]
    assert list(lab[400:]) == m["grid20_tg_erlbm065"]
    lab, _, _ = E().map_run(E().MAP_OBSTACLE, None, precision=E().FP64, n_i=20, n_j=20)
    assert list(lab) == m["grid20_obstacle"]


def test_fp32_shifted_label_agreement_reported():
    """FP32-shifted labels against the reference's on the same subsample.  Near the stability
    boundary labels depend on rounding (FP32 cannot grow instabilities slower than its resolution),
    so this checks a floor and prints the figure."""
    m = ref()
    pts = [tuple(p) for p in m["tg_points"]]
    lab, _, _ = E().map_run(E().MAP_TAYLOR_GREEN, pts, precision=E().FP32_SHIFTED, op=0, tau_nh=0.65)
    agree_tg = np.mean(lab == np.array(m["tg_reg"] + m["tg_erlbm065"]))
    opts = [tuple(p) for p in m["obstacle_points"]]
    lab, _, _ = E().map_run(E().MAP_OBSTACLE, opts, precision=E().FP32_SHIFTED)
    agree_ob = np.mean(lab == np.array(m["obstacle"]))
    print(f"FP32-shifted label agreement with the reference: TG {agree_tg:.4f}, obstacle {agree_ob:.4f}")
    assert agree_tg >= 0.93 and agree_ob >= 0.92
