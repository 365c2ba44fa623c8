"""Host-side logic of the library that runs without a GPU: the C ABI's exported symbols and its
argument checks, the program inputs (initial fields, geometries, map axes) against the oracle, and
the sharding of map points over ranks (gloo, world size 2)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def E():
    import erlbm_gb300 as m
    return m


def declared_functions():
    src = open(os.path.join(ROOT, "include", "erlbm_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(erlbm_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_function():
    lib = E().lib()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_argument_checks_before_any_device_work():
    m = E()
    with pytest.raises(m.ErlbmError) as ei:
        m.Lattice(7, 4, 4)
    assert ei.value.code == -1
    with pytest.raises(m.ErlbmError) as ei:
        m.Lattice(9, 4, 4, 2)  # D2Q9 needs nz = 1
    assert ei.value.code == -1
    with pytest.raises(m.ErlbmError) as ei:
        m.Lattice(19, 4, 4, 1, op=m.OP_MRT)  # coll_MRT is a D2Q9 operator
    assert ei.value.code == -6
    with pytest.raises(ValueError):
        m.operator_from_name("trt")
    assert [m.operator_from_name(n) for n in ("bgk", "mrt", "reg", "erlbm")] == [1, 2, 3, 4]
    for kw in (dict(radius=-1), dict(late_fraction=1.5), dict(probe_stride=-1), dict(max_passes=-1)):
        with pytest.raises(m.ErlbmError) as ei:
            m.map_run_refined(m.MAP_OBSTACLE, n_i=4, n_j=4, **kw)
        assert ei.value.code == -1


def test_program_inputs_equal_oracle():
    m = E()
    for q in (9, 19):
        for variant in (0, 1):
            for neq in (True, False):
                a = m.init_taylor_green(q, 24, 0.05, 0.6, neq=neq, variant=variant)
                b = O.init_taylor_green(q, 24, 0.05, 0.6, neq=neq, variant=variant)
                assert np.array_equal(a, b)
    assert np.array_equal(m.init_double_shear(64), O.init_double_shear(64))
    assert np.array_equal(m.equilibrium(19, 0.1, -0.05, 0.02, 1.01), O.equilibrium(19, 0.1, -0.05, 0.02, 1.01))
    for sx, sy in ((1, 1), (2, 3), (4, 4)):
        a, b = m.obstacle_geometry(sx, sy), O.obstacle_geometry(sx, sy)
        assert a[:2] == b[:2] and np.array_equal(a[2], b[2])
    nx, ny, solid = m.obstacle_geometry()
    assert (nx, ny, int((solid == 0).sum())) == (22, 12, 232)
    for (i, j) in ((0, 0), (399, 399), (17, 233)):
        assert m.tg_map_params(i, j, 400, 400, 4, 0.65) == O.tg_map_params(i, j, 400, 400, 4, 0.65)
        assert m.tg_map_params(i, j, 400, 400, 3, 0.65)[2] == 1.0
        assert m.obstacle_map_params(i, j) == O.obstacle_map_params(i, j, 400, 400, 0.1)
    f = O.init_taylor_green(9, 32, 2 / 32, 0.62)
    assert np.array_equal(m.taylor_green_error(9, 32, f, 2 / 32, 0.04, 7), O.taylor_green_error(9, 32, f, 2 / 32,
                                                                                                 0.04, 7))


def test_shard_unshard_roundtrip():
    from erlbm_gb300.sharding import shard, unshard
    pts = [(i, j) for i in range(7) for j in range(5)]
    for world in (1, 2, 3, 8):
        parts = [np.array([p[0] * 100 + p[1] for p in shard(pts, r, world)]) for r in range(world)]
        assert list(unshard(parts, len(pts), world)) == [p[0] * 100 + p[1] for p in pts]


def _gloo_worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from erlbm_gb300.sharding import map_run_sharded
    pts = [(i, j) for i in range(0, 400, 57) for j in range(0, 400, 91)]

    def oracle_map(kind, points, op, tau_nh, max_steps):
        """The oracle in map_run's place (no GPU here): same call, same result layout (op = 0: all RLBM
        results, then all E-RLBM results)."""
        ops = [O.OP_REG, O.OP_EXTREG] if op == 0 else [op]
        res = [O.tg_map(points, op=o, tau_nh=tau_nh if o == O.OP_EXTREG else 1.0, max_steps=max_steps, threads=1)
               for o in ops]
        return tuple(np.concatenate([r[k] for r in res]) for k in range(3))

    # the same call bench.py makes on each GPU rank, with the oracle as the map
    lab, dec, mg = map_run_sharded(1, pts, map_fn=oracle_map, op=0, tau_nh=0.65, max_steps=1500)
    if rank == 0:
        ref = oracle_map(1, pts, 0, 0.65, 1500)
        out.put((np.array_equal(lab, ref[0]) and lab.dtype == ref[0].dtype, np.array_equal(dec, ref[1]),
                 np.array_equal(mg, ref[2])))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_map_gloo_world2():
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_gloo_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = q.get(timeout=240)
    for p in ps:
        p.join(timeout=60)
    assert res == (True, True, True)


def test_read_geo_equals_oracle_and_reference(tmp_path):
    """erlbm_read_geo (host code of the library) against read_geo's geometry.ini from the reference
    library (tests/golden) and the oracle, with and without added layers and walls."""
    import os
    m = E()
    from oracle import oracle as O
    v = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_vectors.npz"))
    path = tmp_path / "geo.vtk"
    path.write_bytes(v["geo_file"].tobytes())
    for pin, pout, wall in ((0, 0, 1), (2, 3, 1), (2, 3, 0)):
        nx, ny, nz, solid = m.read_geo(str(path), pin, pout, bool(wall))
        assert (nx, ny, nz) == (9 + pin + pout, 5, 2)
        assert np.array_equal(solid == 0, v[f"geo_ini_{pin}_{pout}_{wall}"] != 0)
        assert np.array_equal(solid, O.read_geo(str(path), pin, pout, bool(wall))[3])
    with pytest.raises(m.ErlbmError):
        m.read_geo(str(tmp_path / "missing.vtk"))


def test_channel_bench_geometry_fits_the_parabolic_inlet():
    """bench.py's channel workload: walls on all four sides and a cylinder; every column holds at
    most ny - 2 fluid nodes, the parabolic profile's L, so erlbm_step accepts the inlet."""
    import bench
    for ny in (64, 128, 512):
        nx, solid = bench.channel_geometry(ny)
        s = solid.reshape(ny, nx)
        assert nx == 4 * ny and s[:, 0].all() and s[:, -1].all() and s[0, :].all() and s[-1, :].all()
        assert (1 - s).sum(axis=0).max() == ny - 2
        assert s[ny // 2, ny] == 1 and s[ny // 2, 2 * ny] == 0  # the cylinder, and open channel behind it


def test_bench_reads_its_committed_measurements():
    """The bench line's `roofline.traffic` of the channel and the t* = 1 errors come from committed
    ncu and accuracy measurements: the files parse, the channel traffic scales with the box from the
    captured 4096 x 1024 channel, and the errors say which FP32 form meets the 1e-5 target."""
    import bench
    t = bench.channel_traffic(4096, 1024)
    assert t is not None and 72 * 4096 * 1024 * 0.5 < t < 72 * 4096 * 1024 * 1.5
    assert abs(bench.channel_traffic(2048, 512) - t / 4) < 1
    acc = bench.accuracy_t1()
    assert acc["fp32"]["met"] is False and acc["fp32"]["L2048"] > 1e-5
    assert acc["pair"]["met"] is True and acc["pair"]["L2048"] < 1e-5
    assert bench.ncu_traffic(2048, "fp32_x3a") > 0 and bench.fp64_ops_per_lu(2048) == 169


def test_bench_launch_count_follows_erlbm_step():
    """bench.py's launch count per call of n steps: graph blocks of 64 steps (66 with three steps per
    launch), then multi-step launches, then single steps -- the decomposition erlbm_step makes."""
    import bench
    assert bench.launches_of(1000, 1) == 1000
    assert bench.launches_of(1000, 2) == 500
    assert bench.launches_of(1000, 3) == 15 * 22 + 3 + 1  # 990 in graphs, 9 in three launches, 1 single
    assert bench.launches_of(999, 3) == 15 * 22 + 3
    assert bench.launches_of(65, 2) == 32 + 1
    assert bench.launches_of(2, 3) == 2


def test_autotune_cache_survives_concurrent_writers(tmp_path, monkeypatch):
    """Processes storing tuning results at once (the ranks of one job) leave a readable cache that
    holds one of the writers' complete entries."""
    import multiprocessing as mp
    monkeypatch.setenv("ERLBM_TUNE_CACHE", str(tmp_path / "tune.json"))
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_store_many, args=(str(tmp_path / "tune.json"), r)) for r in range(4)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    from erlbm_gb300 import autotune
    d = autotune._load()
    assert d and all(isinstance(v, dict) and v["rank"] in range(4) for v in d.values())


def _store_many(path, rank):
    import os
    os.environ["ERLBM_TUNE_CACHE"] = path
    from erlbm_gb300 import autotune
    for k in range(50):
        autotune._store(f"key{k % 5}", {"rank": rank, "k": k})


STRUCTS = [("erlbm_desc", "Desc"), ("erlbm_bc", "BC"), ("erlbm_checks", "Checks"),
           ("erlbm_run_result", "RunResult"), ("erlbm_map_desc", "MapDesc"), ("erlbm_refine_desc", "RefineDesc"),
           ("erlbm_batch_desc", "BatchDesc"), ("erlbm_run_spec", "RunSpec"), ("erlbm_batch_result", "BatchResult"),
           ("erlbm_server_desc", "ServerDesc"), ("erlbm_request", "Request"), ("erlbm_result", "Result")]


def test_ctypes_structs_match_the_header(tmp_path):
    """Every struct of include/erlbm_gb300.h that the Python binding mirrors has the same size and the
    same field names and offsets in both (a C program compiled against the header prints them)."""
    import os
    import shutil
    import subprocess
    from erlbm_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    include = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "erlbm_gb300.h"', "int main(void) {"]
    for cname, pyname in STRUCTS:
        cls = getattr(_lib, pyname)
        lines.append(f'    printf("{pyname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'    printf("{pyname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", f"-I{include}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, pyname in STRUCTS:
        cls = getattr(_lib, pyname)
        assert got[(pyname, "size")] == C.sizeof(cls), pyname
        for fname, _ in cls._fields_:
            assert got[(pyname, fname)] == getattr(cls, fname).offset, (pyname, fname)


def test_product_never_loads_the_oracle():
    """The package is the product and the oracle is only the checker: importing erlbm_gb300 and loading
    its library in a fresh interpreter imports no oracle module and maps no oracle library, and no source
    of the package names the oracle."""
    import subprocess
    import sys
    code = ("import sys, erlbm_gb300 as m; m.lib(); "
            "maps = open('/proc/self/maps').read() if sys.platform.startswith('linux') else ''; "
            "print(any(k == 'oracle' or k.startswith('oracle.') for k in sys.modules), 'erlbm_oracle' in maps)")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, check=True)
    assert out.stdout.split() == ["False", "False"], out.stdout
    pkg = os.path.join(ROOT, "erlbm_gb300")
    for d, _, files in os.walk(pkg):
        if "_build" in d:
            continue
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                assert "oracle" not in open(os.path.join(d, f)).read(), f


def test_reference_arm_prints_the_contract_line():
    """bench.py --impl reference times the reference's CPU path (the reference compiled from its sources
    where present, else the oracle port) without a GPU and prints one JSON line with the arm's keys: the
    metric of the engine's arm, a cpu_baseline describing the run and an e2e with no copies."""
    import json
    import subprocess
    import sys
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"],
                         cwd=ROOT, capture_output=True, text=True, check=True, timeout=600)
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "MLUPS" and line["unit"] == "MLUPS"
    assert line["value"] > 0 and line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 3
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["unit"] == "MLUPS" and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["L"] == 2048


def test_reference_arm_under_torchrun_prints_once():
    """Launched as the multi-GPU bench is (torchrun, two ranks), the reference arm runs on rank 0 alone:
    one JSON line, n_gpus = 2, and every rank exits 0."""
    import json
    import socket
    import subprocess
    import sys
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                          "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
                          "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"],
                         cwd=ROOT, capture_output=True, text=True, check=True, timeout=600)
    lines = [json.loads(x) for x in out.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, out.stdout
    assert lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2 and lines[0]["value"] > 0
