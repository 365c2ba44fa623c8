"""The drop-in from compiled C++: tests/drivers/erlbm_driver.cpp includes include/erlbm_gb300.h, links
liberlbm_gb300.so and runs two of the reference's loops through the C ABI (no Python in the loop):
the obstacle map's roda_ponto (main_stability-map_obstacle.cpp:75-123: boundary planes, collision,
density check every step) and the double shear layer's interval loop (main_double-shear-layer.cpp:
162-230: steps, then the kinetic energy of the post-collision populations).  The labels equal those of
the reference's own roda_ponto (tests/golden/reference_maps_20x20.json), the energies the oracle's."""
import json
import os
import shutil
import subprocess

import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from erlbm_gb300 import build
    lib = build.build()
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("driver") / "erlbm_driver")
    libdir = os.path.dirname(lib)
    subprocess.run([cxx, "-std=c++17", "-O2", os.path.join(HERE, "drivers", "erlbm_driver.cpp"),
                    f"-I{os.path.join(ROOT, 'include')}", f"-L{libdir}", "-lerlbm_gb300", f"-Wl,-rpath,{libdir}",
                    "-o", exe], check=True)
    return exe


def run(exe, *args):
    out = subprocess.run([exe, *map(str, args)], capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr
    return [json.loads(l) for l in out.stdout.splitlines() if l.strip()]


def test_obstacle_roda_ponto_from_cpp_matches_reference_labels(driver):
    with open(os.path.join(HERE, "golden", "reference_maps_20x20.json")) as f:
        gold = json.load(f)
    label = {tuple(p): l for p, l in zip(gold["obstacle_points"], gold["obstacle"])}
    for i, j in ((0, 0), (20, 0), (140, 140), (60, 160)):
        (r,) = run(driver, "obstacle", i, j)
        assert r["label"] == label[(i, j)], r
        if r["label"] == 0:
            assert r["steps"] == r["n_steps"]


def test_dsl_interval_loop_from_cpp_matches_oracle_energies(driver):
    L, interval, n = 64, 50, 3
    got = run(driver, "dsl", L, interval, n)
    lat = O.Lattice(9, L, L, 1, None, 0.5 + 3 * (1 / 32) * L / 80000, 0.65, O.OP_EXTREG)
    lat.set(O.init_double_shear(L))
    for k, r in enumerate(got, 1):
        lat.step(interval)
        assert r["step"] == k * interval
        assert r["energy"] == lat.kinetic_energy(1), (r, lat.kinetic_energy(1))
