#!/usr/bin/env python
"""bench.py -- throughput of the E-RLBM collide-stream hot path on GB300.

Workload (one bench step): `inner` steps of the double shear layer (D2Q9, E-RLBM tau_nh = 0.65,
Re = 80000, U0 = 1/32, lambda = 80, epsilon = 0.05; main_double-shear-layer.cpp) on an L x L
periodic lattice, L = 2048 by default, FP32-shifted populations.  The metric is MLUPS (million
lattice updates per second); `value` is device-timed with CUDA events on the stream the kernels
run on, with the populations already resident in HBM.  The working set (2 x 9 x 4 B x L^2 =
302 MB at L = 2048) is larger than the 129 MB L2, so no flush is needed between steps.

`e2e` is the same metric through the C ABI as a caller uses it: each bench step copies the
initial populations from pinned host memory (erlbm_set_populations, AoS doubles), runs `inner`
steps (erlbm_step) and reads the kinetic energy back (erlbm_kinetic_energy), wall-clock timed.

`fp64` is the plain FP64 path on the same lattice, the drop-in that reproduces the reference's FP64
results bit for bit: device-timed MLUPS, its own `e2e` through the C ABI, and its roofline against
the GPU's FP64 add / multiply rate (measured in the run) and against the HBM copy peak.  It is the
like-for-like comparison with the reference arm, which computes in FP64 too.

`cpu_baseline` times the CPU restatement of the reference's algorithm (oracle/, AoS + push map,
OpenMP over all host cores) on a bounded sample of the same workload.  `--impl reference` runs the
reference's own CPU code when it could be compiled from its sources here (oracle/_ref), otherwise
that same restatement, and prints the same JSON line with "impl": "reference".

Multi-GPU: one lattice does not shard, so N GPUs run N independent replicas (weak scaling).

Other workloads (--workload; the default is the one above):
  tg-map, obstacle-map   stability maps (main_stability-map_*.cpp) on an evenly spaced P x P subset
                         of the 400 x 400 grid; one bench step = one batched map launch per GPU; runs/s.
                         The Taylor-Green map runs every point with RLBM and with E-RLBM.  Under
                         torchrun the points are sharded over the ranks (weak in GPUs, strong in points).
  serve                  a seeded Poisson stream of mixed requests (Taylor-Green D2Q9 L = 32..512,
                         map points, obstacle channels scaled 1-4x, 3-D Taylor-Green 32^3 / 64^3;
                         FP32 or FP64; budgets 1..10000 steps) through the request server; runs/s
                         with p50 / p99 latency, beside the plain path (one run at a time, FP64,
                         one launch per step) on an evenly strided sample of the same stream.
  snapshot               the double shear layer's output at an interval (main_double-shear-layer.cpp:
                         187-208): kinetic energy, rec_velocity and rec_vorticity as ASCII VTK, from
                         the resident populations (fields on the device); snapshots/s, wall-clock,
                         beside the CPU restatement writing the same files from host populations.
  channel                a D2Q9 channel (the library's channel boundaries, Boundary_conditions.cpp:
                         456-806): walls, a circular cylinder, parabolic inlet, convective outlet,
                         nx = 4 ny (ny = L / 2: 4096 x 1024 at L = 2048, whose two population buffers
                         exceed L2 in FP32); `inner` steps per bench step; MLUPS over fluid nodes.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

# before any CUDA context exists: the server's resident loops need their own hardware work queues
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_LU = {"fp32": 2 * 9 * 4, "fp64": 2 * 9 * 8, "pair": 2 * 9 * 8}


# DSL operators as main_double-shear-layer.cpp takes them (--collision; tau_nh = 1 for reg, :89):
# name -> (op code, tau_nh, label)
DSL_OPS = {"erlbm": (4, 0.65, "E-RLBM tau_nh=0.65"), "reg": (3, 1.0, "RLBM"), "bgk": (1, 0.65, "BGK"),
           "mrt": (2, 0.65, "MRT")}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--L", type=int, default=2048)
    p.add_argument("--inner", type=int, default=1000, help="LBM steps per bench step")
    p.add_argument("--inner-fp64", type=int, default=100,
                   help="dsl: LBM steps per bench step of the plain FP64 block beside the FP32-shifted line")
    p.add_argument("--precision", default="fp32", choices=["fp32", "fp64", "pair", "refined"],
                   help="pair (dsl): the compensated FP32 form (float-pair populations, float-float collision); "
                        "refined (map workloads): the whole map-points x map-points grid screened in FP32 with "
                        "the boundary points re-run in FP64")
    p.add_argument("--cpu-seconds", type=float, default=10.0, help="target length of the CPU baseline sample")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-extras", action="store_true")
    p.add_argument("--workload", default="dsl",
                   choices=["dsl", "tg-map", "obstacle-map", "serve", "snapshot", "channel"])
    p.add_argument("--op", default="erlbm", choices=list(DSL_OPS),
                   help="dsl: collision operator (main_double-shear-layer.cpp --collision)")
    p.add_argument("--map-points", type=int, default=100, help="P: P x P map points per bench step")
    p.add_argument("--max-steps", type=int, default=0, help="cap on map run budgets (0 = the reference's)")
    p.add_argument("--requests", type=int, default=400, help="serve: requests in the stream")
    p.add_argument("--rate", type=float, default=2000.0, help="serve: mean arrivals per second")
    p.add_argument("--plain-requests", type=int, default=24, help="serve: sampled requests run on the plain path")
    p.add_argument("--team-ctas", type=int, default=0,
                   help="serve: CTAs of each resident team loop (0 = one per SM; -1 = no team loop, those "
                        "requests take the stream lane)")
    p.add_argument("--team-max-nodes", type=int, default=0,
                   help="serve: largest lattice the team loops take (0 = the server's default, 2^19)")
    p.add_argument("--single-runs", action="store_true",
                   help="serve: also time single requests alone on the team loop and on the stream lane")
    return p.parse_args()


def tau_of(L: int) -> float:
    # main_double-shear-layer.cpp:307: tau = 1/2 + 3 U0 L / Re
    return 0.5 + 3.0 * (1.0 / 32.0) * L / 80000.0


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def launches_of(n: int, per: int) -> int:
    """Kernel launches of erlbm_step(n) on a lattice whose last step was a collision: blocks of 64 steps
    (66 with three steps per launch) replayed as graphs, then multi-step launches, then single steps."""
    g = 66 if per == 3 else 64
    count, s = 0, 0
    while s < n:
        if n - s >= g:
            count, s = count + g // per, s + g
        elif per > 1 and n - s >= per:
            count, s = count + 1, s + per
        else:
            count, s = count + 1, s + 1
    return count


def ncu_traffic(L: int, precision: str):
    """DRAM bytes per launch from the committed ncu summary of the same kernel ("fp32", "fp64",
    "fp32_x2" or "fp32_x3" for the two- and three-step kernels), scaled to L."""
    path = os.path.join(ROOT, "profiles", "dsl_periodic_d2q9_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        rec = d[precision]
        return rec.get("dram_bytes_per_node_per_launch", rec.get("dram_bytes_per_lu")) * L * L
    except Exception:
        return None


def channel_traffic(nx: int, ny: int):
    """DRAM bytes per launch of the FP32 channel kernel from its committed ncu summary, scaled by the
    box (the capture is of the bench's own 4096 x 1024 channel)."""
    try:
        with open(os.path.join(ROOT, "profiles", "channel_step_traffic.json")) as f:
            rec = json.load(f)["fp32"]
        return (rec["dram_bytes_read"] + rec["dram_bytes_write"]) * (nx * ny) / (rec["nx"] * rec["ny"])
    except Exception:
        return None


class Clocks:
    """nvidia-smi sampling during the timed region (clocks and throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.fh = open(self.path, "w")
        self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                     stderr=subprocess.DEVNULL)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx = float(parts[2])
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------------
# CPU legs (the only places bench.py executes oracle/)
# ------------------------------------------------------------------------------------------------

class CpuDsl:
    """The reference's CPU algorithm for the double shear layer on this host's cores: the reference
    library compiled from its sources (oracle/_ref, only where it was built) or the oracle's
    restatement of it.  run(n) advances n steps and returns the seconds they took."""

    def __init__(self, L: int, prefer_reference: bool, op_name: str = "erlbm"):
        from oracle import oracle as O
        self.L = L
        self.threads = os.cpu_count() or 1
        self.tau = tau_of(L)
        self.op, self.tnh, self.label = DSL_OPS[op_name]
        self.f0 = O.init_double_shear(L)
        self.kind = "port"
        self.overhead = 0.0
        if prefer_reference and O.ref_available(9):
            import ctypes as C
            lib = O.load_ref(9)
            fn = lib.ref9_run_threads
            fn.restype = C.c_int
            fn.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_void_p,
                           C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                           C.c_int]
            self._fn = fn
            self.kind = "reference"
            # each harness call sets the lattice up and copies its output: that fixed cost (a 1-step call
            # less one step, the step time taken from a 1-step and a 5-step call) is taken out of every
            # sample.  The first call pays one-time costs (threads, pages) and is not used; the step time
            # is at least a tenth of the 5-step call's, so that noise cannot make it vanish.
            self._call(1)
            t1 = self._call(1)
            t5 = self._call(5)
            self.step_s = max((t5 - t1) / 4, t5 / 10, 1e-6)
            self.overhead = max(0.0, t1 - self.step_s)
        else:
            self._lat = O.Lattice(9, L, L, 1, None, self.tau, self.tnh, self.op)
            self._lat.set(self.f0)

    def _call(self, n: int) -> float:
        t = time.perf_counter()
        self._fn(self.L, self.L, 1, None, self.op, self.tau, self.tnh, self.f0.ctypes.data, n, -1, 0.0, -1, 1.0,
                 None, None, None, self.threads)
        return time.perf_counter() - t

    def run(self, n: int) -> float:
        if self.kind == "reference":
            return max(self._call(n) - self.overhead, 1e-9)
        t = time.perf_counter()
        self._lat.step(n, threads=self.threads)
        return time.perf_counter() - t

    def steps_for(self, seconds: float) -> int:
        """LBM steps that take about `seconds` here (from a short probe)."""
        t1 = self.step_s if self.kind == "reference" else self.run(2) / 2
        return max(2, min(2000, int(seconds / max(t1, 1e-6))))

    def describe(self, n: int) -> str:
        return (f"double shear layer D2Q9 {self.label} FP64, L={self.L}, {n} steps, "
                f"{self.threads} OpenMP threads")


def cpu_sample(L: int, seconds: float, prefer_reference: bool, op_name: str = "erlbm"):
    """One bounded sample (about `seconds` of CPU work) of the reference's CPU algorithm."""
    cpu = CpuDsl(L, prefer_reference, op_name)
    n = cpu.steps_for(seconds)
    dt = cpu.run(n)
    return {"value": L * L * n / dt / 1e6, "unit": "MLUPS", "cores": cpu.threads, "kind": cpu.kind,
            "sample": cpu.describe(n)}


def run_reference(args):
    """The reference arm: the reference's CPU path on the host cores.  Every bench step runs the same
    bounded number of LBM steps (chosen once, so that the whole run takes a few minutes), and the line
    reports exactly that count and the measured time per bench step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    W, K, L = args.warmup, args.steps, args.L
    cpu = CpuDsl(L, True, args.op)
    per = max(1.0, min(8.0, 120.0 / max(1, K + W)))  # seconds of CPU work per bench step
    n = cpu.steps_for(per)
    for _ in range(W):
        cpu.run(max(1, n // 4))
    times = [cpu.run(n) for _ in range(K)]
    total = sum(times)
    v = L * L * n * K / total / 1e6
    cb = {"value": v, "unit": "MLUPS", "cores": cpu.threads, "kind": cpu.kind,
          "sample": cpu.describe(n) + f" per bench step, {K} bench steps"}
    line = {"metric": "MLUPS", "value": v, "unit": "MLUPS", "n_gpus": args.gpus, "steps": K, "warmup": W,
            "ms_per_step": total / K * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (double shear layer initial condition)",
            "config": {"workload": f"double shear layer D2Q9 {DSL_OPS[args.op][2]} Re=80000 L={L}", "L": L,
                       "lbm_steps_per_step": n, "precision": "fp64 (reference CPU path)",
                       "warmup_lbm_steps_per_step": max(1, n // 4)},
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------------------
# GPU leg
# ------------------------------------------------------------------------------------------------

def run_ours(args):
    import numpy as np
    import torch
    import erlbm_gb300 as E

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()

    L, inner, K, W = args.L, args.inner, args.steps, args.warmup
    prec = {"fp32": E.FP32_SHIFTED, "fp64": E.FP64, "pair": E.FP32_PAIR}[args.precision]
    tau = tau_of(L)
    f0 = E.init_double_shear(L)
    stream = torch.cuda.Stream()
    op, tnh, op_label = DSL_OPS[args.op]
    lat = E.Lattice(9, L, L, 1, None, tau, tnh, op, prec)
    shape = None
    if args.precision == "fp32" and L % 128 == 0:
        from erlbm_gb300 import autotune  # launch shape chosen by measurement (cached), outside the timed region
        shape = autotune.apply_periodic(lat)
    lat.set_stream(stream.cuda_stream)
    lat.set_populations(f0)
    lat.step(1)  # the first step collides the given populations in place; later ones are fused
    for _ in range(W):
        lat.step(inner)
    lat.sync()

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-timed region -------------------------------------------------------------------
    barrier()
    clocks = Clocks(dev)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(K):
        lat.step(inner)
    ev1.record(stream)
    stream.synchronize()
    barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    per = 3 if (shape and shape.get("three_step")) else (2 if (shape and shape.get("two_step")) else 1)
    wide = bool(per == 3 and shape.get("wide_strips"))
    launches = K * launches_of(inner, per)
    value = world * L * L * inner * K / (ms / 1e3) / 1e6
    launch_ms = ms / launches
    algo_bytes = BYTES_PER_LU[args.precision] * L * L
    peak, peak_kind = peaks()
    achieved = algo_bytes / (launch_ms / 1e3) / 1e9

    # ---- end to end through the C ABI with host buffers ------------------------------------------
    pinned = torch.empty(f0.size, dtype=torch.float64, pin_memory=True)
    pinned.numpy()[:] = f0
    host = pinned.numpy()
    for _ in range(max(1, min(W, 2))):
        lat.set_populations(host)
        lat.step(inner)
        lat.kinetic_energy(E.STAGE_POST_COLLISION)
    barrier()
    t0 = time.perf_counter()
    for _ in range(K):
        lat.set_populations(host)
        lat.step(inner)
        lat.kinetic_energy(E.STAGE_POST_COLLISION)
    t_e2e = time.perf_counter() - t0
    if dist:
        t = torch.tensor([t_e2e], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())
    e2e = {"value": world * L * L * inner * K / t_e2e / 1e6, "unit": "MLUPS", "h2d_bytes_per_step": int(f0.nbytes),
           "d2h_bytes_per_step": 8}

    lat.close()
    extras, fp64, pair = {}, None, None
    if not args.no_extras and rank == 0:
        extras = gpu_extras(E, torch, L, f0, tau, op, tnh)
        if args.precision == "fp32":
            fp64 = fp64_block(E, torch, L, f0, tau, op, tnh, K, W, args.inner_fp64)
            if args.op in ("erlbm", "reg", "bgk"):  # the compensated form has no MRT
                pair = pair_block(E, torch, L, f0, tau, op, tnh, K, W, 100)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    cpu = None
    if world == 1 and not args.no_cpu:
        cpu = cpu_sample(L, args.cpu_seconds, False, args.op)
    line = {
        "metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32": "f32", "fp64": "f64", "pair": "f32x2"}[args.precision],
        "data": "synthetic (double shear layer initial condition, main_double-shear-layer.cpp:48-66)",
        "config": {"workload": f"double shear layer D2Q9 {op_label} Re=80000 L={L}, "
                               f"{dict(fp32='FP32-shifted', fp64='FP64 plain', pair='compensated FP32 pairs')[args.precision]}",
                   "L": L, "lbm_steps_per_step": inner, "parallelism": f"replicas x{world}",
                   "l2": f"working set {2 * BYTES_PER_LU[args.precision] // 2 * L * L / 1e6:.0f} MB > 129 MB L2, "
                         "no flush",
                   "launch_shape": None if shape is None else {"block_threads": shape["block_threads"],
                                                               "streaming_stores": shape["streaming_stores"],
                                                               "steps_per_launch": per, "wide_strips": wide}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind,
                     "traffic": ncu_traffic(L, "fp32_x3a" if wide else
                                            {1: args.precision, 2: "fp32_x2", 3: "fp32_x3"}[per])
                     if args.op == "erlbm" else None,
                     "algorithmic_bytes_per_launch": algo_bytes, "launch_us": launch_ms * 1e3,
                     "lattice_updates_per_launch": L * L * per,
                     "kernel": (f"k_periodic_d2q9_x3a<{op}>" if wide else
                                {1: f"k_periodic_d2q9<{op}>", 2: f"k_periodic_d2q9_x2s<{op}>",
                                 3: f"k_periodic_d2q9_x3s<{op}>"}[per])
                     if args.precision == "fp32" else (f"k_step<PrecExact64,9,{op}>" if args.precision == "fp64"
                                                       else f"k_step_pair<{op}>"),
                     # the update rate against the roofline of one step per launch, where every
                     # update reads and writes each population once (2 Q sizeof(real) bytes): the
                     # multi-step kernels move a half or a third of those bytes, so this fraction can exceed 1
                     "one_step_equivalent": {"bytes_per_update": BYTES_PER_LU[args.precision],
                                             "gbs": value * 1e6 * BYTES_PER_LU[args.precision] / 1e9,
                                             "frac": value * 1e6 * BYTES_PER_LU[args.precision] / 1e9 / peak}},
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if fp64:
        line["fp64"] = fp64
    if pair:
        line["pair"] = pair
    if extras:
        acc = accuracy_t1()
        if acc and args.precision == "fp32":
            extras["fp32_vs_fp64_rel_l2_velocity_at_t1"] = acc.get("fp32")
        line["extras"] = extras
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def fp64_ops_per_lu(L: int):
    """FP64 add and multiply operations per lattice update of the plain kernel, from the committed ncu
    instruction counts of the same kernel (profiles/dsl_periodic_d2q9_traffic.json, "fp64")."""
    path = os.path.join(ROOT, "profiles", "dsl_periodic_d2q9_traffic.json")
    try:
        with open(path) as f:
            return float(json.load(f)["fp64"]["fp64_ops_per_lu"])
    except Exception:
        return None


def time_lattice(E, torch, L, f0, tau, op, tnh, K, W, inner, prec):
    """One DSL lattice in precision `prec`: device-timed MLUPS over K bench steps of `inner` LBM steps,
    and the same end to end through the C ABI (populations from pinned host memory, steps, energy
    back).  Returns (MLUPS, ms per bench step, us per launch, e2e MLUPS)."""
    s = torch.cuda.Stream()
    with E.Lattice(9, L, L, 1, None, tau, tnh, op, prec) as lat:
        lat.set_stream(s.cuda_stream)
        lat.set_populations(f0)
        lat.step(1)
        for _ in range(W):
            lat.step(inner)
        lat.sync()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        for _ in range(K):
            lat.step(inner)
        b.record(s)
        s.synchronize()
        ms = a.elapsed_time(b)
        value = L * L * inner * K / (ms / 1e3) / 1e6
        pinned = torch.empty(f0.size, dtype=torch.float64, pin_memory=True)
        pinned.numpy()[:] = f0
        host = pinned.numpy()
        lat.set_populations(host)
        lat.step(inner)
        lat.kinetic_energy(E.STAGE_POST_COLLISION)
        t0 = time.perf_counter()
        for _ in range(K):
            lat.set_populations(host)
            lat.step(inner)
            lat.kinetic_energy(E.STAGE_POST_COLLISION)
        t_e2e = time.perf_counter() - t0
    return value, ms / K, ms / (K * inner) * 1e3, L * L * inner * K / t_e2e / 1e6


def fp64_block(E, torch, L, f0, tau, op, tnh, K, W, inner):
    """The plain FP64 path (bit-identical to the reference) on the same lattice: device-timed and end to
    end, with its roofline against this GPU's FP64 add / multiply rate (measured here with
    erlbm_fp64_rate) and against the HBM copy peak."""
    value, ms_step, launch_us, e2e = time_lattice(E, torch, L, f0, tau, op, tnh, K, W, inner, E.FP64)
    rate = E.fp64_rate()
    ops = fp64_ops_per_lu(L)
    hbm, hbm_kind = peaks()
    return {
        "lbm_steps_per_step": inner, "steps": K, "warmup": W,
        "value": value, "unit": "MLUPS", "dtype": "f64", "ms_per_step": ms_step,
        "kernel": f"k_step<PrecExact64,9,{op}>",
        "e2e": {"value": e2e, "unit": "MLUPS", "h2d_bytes_per_step": int(f0.nbytes), "d2h_bytes_per_step": 8},
        "roofline": {"bound": "fp64", "unit": "Gop/s",
                     "achieved": None if ops is None else ops * value * 1e6 / 1e9,
                     "peak": rate / 1e9, "peak_kind": "measured in this run (erlbm_fp64_rate: unfused DADD/DMUL)",
                     "frac": None if ops is None else ops * value * 1e6 / rate,
                     "fp64_ops_per_lu": ops, "launch_us": launch_us},
        "hbm": {"bytes_per_lu": BYTES_PER_LU["fp64"], "achieved_gbs": value * 1e6 * BYTES_PER_LU["fp64"] / 1e9,
                "peak_gbs": hbm, "frac": value * 1e6 * BYTES_PER_LU["fp64"] / 1e9 / hbm, "peak_kind": hbm_kind},
    }


def pair_block(E, torch, L, f0, tau, op, tnh, K, W, inner):
    """The compensated FP32 form (float-pair populations, float-float collision), the FP32 variant that
    meets the 1e-5 velocity-error target, on the same lattice: device-timed and end to end, against
    the HBM copy peak at its 144 B per update, with its measured error at t* = 1."""
    value, ms_step, launch_us, e2e = time_lattice(E, torch, L, f0, tau, op, tnh, K, W, inner, E.FP32_PAIR)
    hbm, hbm_kind = peaks()
    out = {
        "lbm_steps_per_step": inner, "steps": K, "warmup": W,
        "value": value, "unit": "MLUPS", "dtype": "f32x2", "ms_per_step": ms_step, "kernel": f"k_step_pair<{op}>",
        "e2e": {"value": e2e, "unit": "MLUPS", "h2d_bytes_per_step": int(f0.nbytes), "d2h_bytes_per_step": 8},
        "roofline": {"bound": "hbm", "unit": "GB/s", "achieved": value * 1e6 * BYTES_PER_LU["pair"] / 1e9,
                     "peak": hbm, "frac": value * 1e6 * BYTES_PER_LU["pair"] / 1e9 / hbm, "peak_kind": hbm_kind,
                     "bytes_per_lu": BYTES_PER_LU["pair"], "launch_us": launch_us},
    }
    acc = accuracy_t1()
    if acc:
        out["rel_l2_velocity_vs_fp64_at_t1"] = acc.get("pair")
    return out


def accuracy_t1():
    """Relative L2 velocity errors against FP64 at t* = 1 of the double shear layer (65 537 steps at
    L = 2048, too long for a bench step), from the committed measurement (programs.precision_error)."""
    try:
        with open(os.path.join(ROOT, "profiles", "accuracy_t1.json")) as f:
            return json.load(f)
    except Exception:
        return None


def gpu_extras(E, torch, L, f0, tau, op, tnh):
    """The FP32-shifted velocity error against the plain FP64 path after a short common run."""
    import numpy as np
    out = {}
    n = 1 + 10 + 200
    with E.Lattice(9, L, L, 1, None, tau, tnh, op, E.FP64) as l64:
        l64.set_populations(f0)
        l64.step(n)
        _, u64 = l64.macroscopic(E.STAGE_POST_COLLISION)
    with E.Lattice(9, L, L, 1, None, tau, tnh, op, E.FP32_SHIFTED) as l32:
        l32.set_populations(f0)
        l32.step(n)
        _, u32 = l32.macroscopic(E.STAGE_POST_COLLISION)
    out["fp32_vs_fp64_rel_l2_velocity"] = float(np.linalg.norm(u32 - u64) / np.linalg.norm(u64))
    out["fp32_vs_fp64_steps"] = n
    return out


def map_points(P):
    step = 400 / P
    return [(int(i * step), int(j * step)) for j in range(P) for i in range(P)]


def run_map(args):
    """Map points are independent runs: under torchrun each rank (one GPU) runs a strided share of the
    points and the labels are gathered (erlbm_gb300.sharding.map_run_sharded); `value` is the runs of all
    ranks over the slowest rank's time."""
    import numpy as np
    import torch
    import erlbm_gb300 as E
    from erlbm_gb300.sharding import map_run_sharded
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    kind = E.MAP_TAYLOR_GREEN if args.workload == "tg-map" else E.MAP_OBSTACLE
    refined = args.precision == "refined"
    if refined and world > 1:
        raise SystemExit("the refined map's FP64 passes follow label changes across the whole grid; it runs on one GPU")
    prec = E.FP64 if args.precision == "fp64" else E.FP32_SHIFTED
    pts = map_points(args.map_points)
    P = args.map_points

    def one_map(points):
        if refined:  # the whole P x P grid of the map's axes; refinement needs neighbours
            lab, dec, _, ref, passes = E.map_run_refined(kind, op=op, n_i=P, n_j=P, max_steps=args.max_steps,
                                                         slots=-1, return_passes=True)
            return lab, dec, int(ref.sum()), passes
        lab, dec, _ = map_run_sharded(kind, points, precision=prec, op=op, max_steps=args.max_steps, slots=-1)
        return lab, dec, 0, 0

    op = 0 if kind == E.MAP_TAYLOR_GREEN else E.OP_EXTREG
    nodes = 256 if kind == E.MAP_TAYLOR_GREEN else 232
    from erlbm_gb300 import autotune
    tuned = autotune.tune_map(kind, prec)  # cached after the first run; outside the timed region
    for _ in range(args.warmup):
        E.map_run(kind, pts[: max(1, len(pts) // 8)], precision=prec, op=op, max_steps=args.max_steps, slots=-1)
    if refined:
        autotune.tune_map(kind, E.FP64)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = Clocks(torch.cuda.current_device())
    clocks.start()
    t0 = time.perf_counter()
    runs, lus, n_ref, n_pass = 0, 0, 0, 0
    for _ in range(args.steps):
        lab, dec, nr, npass = one_map(pts)
        runs += len(lab)
        n_ref += nr
        n_pass += npass
        lus += int(np.sum(dec.astype(np.int64))) * nodes
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    clk = clocks.stop()
    if dist:
        t = torch.tensor([dt], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dt = float(t.item())
        dist.destroy_process_group()
        if rank != 0:
            return 0
    value = runs / dt  # the gathered label arrays hold every rank's runs
    line = {"metric": "map runs/s", "value": value, "unit": "runs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if refined else ("f32" if prec else "f64"),
            "data": "synthetic (the reference's map axes)",
            "config": {"workload": f"{args.workload} D3Q19, "
                                   + (f"whole {P}x{P} grid" if refined else f"{P}x{P} points of the 400x400 grid")
                                   + f"{' x {RLBM, E-RLBM}' if op == 0 else ''}, max_steps={args.max_steps}",
                       "precision": args.precision, "slots_per_sm": tuned["slots"],
                       "parallelism": f"points sharded over {world} GPU(s), labels gathered"},
            "lattice_updates_per_s": lus / dt, "roofline": None,
            "e2e": {"value": value, "unit": "runs/s", "h2d_bytes_per_step": len(pts) * 48,
                    "d2h_bytes_per_step": len(pts) * 32},
            "gpu_launches": args.steps + n_pass, "clocks": clk}
    if refined:
        line["refined_fraction"] = n_ref / runs
        line["fp64_passes_per_map"] = n_pass / args.steps
    if not args.no_cpu and world == 1:
        from oracle import oracle as O
        few = pts[:: max(1, len(pts) // 16)]
        t = time.perf_counter()
        if kind == E.MAP_TAYLOR_GREEN:
            O.tg_map(few, op=O.OP_EXTREG, tau_nh=0.65, max_steps=args.max_steps)
        else:
            O.obstacle_map(few, max_steps=args.max_steps)
        ct = time.perf_counter() - t
        line["cpu_baseline"] = {"value": len(few) / ct, "unit": "runs/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{len(few)} of the same points, OpenMP over points"}
    print(json.dumps(line), flush=True)
    return 0


def serve_stream(E, n, rate, seed=20261203):
    """Config-5 request mix: (arrival time, request kwargs) in arrival order."""
    import numpy as np
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    out = []
    for k in range(n):
        kind = int(rng.integers(0, 4))
        prec = [E.FP32_SHIFTED, E.FP64][int(rng.integers(0, 2))]
        steps = int(rng.integers(1, 10001))
        if kind == 0:
            L = int(rng.choice([32, 64, 128, 256, 512]))
            u0 = 2.0 / L
            r = dict(kind=E.REQ_TG2D, precision=prec, op=E.OP_EXTREG, L=L, tau=0.5 + 3 * u0 * L / 50.0, tau_nh=0.65,
                     u0=u0, n_steps=steps)
        elif kind == 1:
            op = [E.OP_REG, E.OP_EXTREG][int(rng.integers(0, 2))]
            u0, tau, tnh = E.tg_map_params(int(rng.integers(0, 400)), int(rng.integers(0, 400)), op=op)
            r = dict(kind=E.REQ_TG_MAP_POINT, precision=prec, op=op, tau=tau, tau_nh=tnh, u0=u0, n_steps=steps)
        elif kind == 2:
            u, tau, tnh = E.obstacle_map_params(int(rng.integers(0, 400)), int(rng.integers(0, 400)))
            r = dict(kind=E.REQ_OBSTACLE, precision=prec, op=E.OP_EXTREG, sx=int(rng.integers(1, 5)),
                     sy=int(rng.integers(1, 5)), tau=tau, tau_nh=tnh, u0=u, n_steps=steps)
        else:
            r = dict(kind=E.REQ_TG3D, precision=prec, op=E.OP_EXTREG, L=int(rng.choice([32, 64])), tau=0.55,
                     tau_nh=0.65, u0=0.05, n_steps=steps)
        out.append((float(t[k]), r))
    return out


def plain_run(E, r):
    """One request on the plain single-lattice path: FP64, one launch per step, one run at a time."""
    import numpy as np
    k = r["kind"]
    if k == E.REQ_TG2D:
        L = r["L"]
        with E.Lattice(9, L, L, 1, None, r["tau"], r["tau_nh"], r["op"], E.FP64) as lat:
            lat.set_populations(E.init_taylor_green(9, L, r["u0"], r["tau"]))
            lat.step(r["n_steps"])
            return lat.kinetic_energy()
    if k == E.REQ_TG_MAP_POINT:
        with E.Lattice(19, 16, 16, 1, None, r["tau"], r["tau_nh"], r["op"], E.FP64) as lat:
            lat.set_populations(E.init_taylor_green(19, 16, r["u0"], r["tau"], poisson=False, neq=False))
            return lat.run(r["n_steps"], None, energy_every=100, energy_factor=2.0)["label"]
    if k == E.REQ_OBSTACLE:
        nx, ny, solid = E.obstacle_geometry(r["sx"], r["sy"])
        with E.Lattice(19, nx, ny, 1, solid, r["tau"], r["tau_nh"], r["op"], E.FP64) as lat:
            lat.set_populations(np.tile(E.equilibrium(19, 0, 0, 0, 1.0), lat.n_fluid))
            return lat.run(r["n_steps"], dict(inlet_x=1, u_in=r["u0"], outlet_x=nx - 2, rho_out=1.0),
                           density_check=True)["label"]
    L = r["L"]
    with E.Lattice(19, L, L, L, None, r["tau"], r["tau_nh"], r["op"], E.FP64) as lat:
        lat.set_populations(np.concatenate([E.init_taylor_green(19, L, r["u0"], r["tau"], poisson=False, neq=False,
                                                                nz=1)] * L))
        lat.step(r["n_steps"])
        return lat.kinetic_energy()


def serve_single_runs(E, args):
    """Wall time (ms) from submission to result of single requests on an otherwise idle server, on the
    team loop and on the stream lane, and of 16 copies of the 64^3 FP64 request submitted together."""
    reqs = {
        "tg3d64_fp64": dict(kind=E.REQ_TG3D, precision=E.FP64, op=E.OP_EXTREG, L=64, tau=0.55, tau_nh=0.65,
                            u0=0.05, n_steps=500),
        "tg2d512_fp64": dict(kind=E.REQ_TG2D, precision=E.FP64, op=E.OP_EXTREG, L=512, tau=0.56, tau_nh=0.65,
                             u0=2 / 512, n_steps=500),
        "tg3d64_fp32": dict(kind=E.REQ_TG3D, precision=E.FP32_SHIFTED, op=E.OP_EXTREG, L=64, tau=0.55, tau_nh=0.65,
                            u0=0.05, n_steps=500),
        "tg2d512_fp32": dict(kind=E.REQ_TG2D, precision=E.FP32_SHIFTED, op=E.OP_EXTREG, L=512, tau=0.56,
                             tau_nh=0.65, u0=2 / 512, n_steps=500),
        "tg2d64_fp64": dict(kind=E.REQ_TG2D, precision=E.FP64, op=E.OP_EXTREG, L=64, tau=0.56, tau_nh=0.65,
                            u0=2 / 64, n_steps=500),
        "obstacle3x3_fp64": dict(kind=E.REQ_OBSTACLE, precision=E.FP64, op=E.OP_EXTREG, sx=3, sy=3, tau=0.52,
                                 tau_nh=0.6, u0=0.05, n_steps=500),
    }
    out = {}
    for lane, team_ctas in (("team", args.team_ctas), ("stream", -1)):
        with E.Server(hbm_budget_bytes=4 << 30, team_ctas=team_ctas, team_max_nodes=args.team_max_nodes) as srv:
            for name, r in reqs.items():
                srv.wait(srv.submit(**dict(r, n_steps=5)), 600.0)
                t = time.perf_counter()
                srv.wait(srv.submit(**r), 600.0)
                out.setdefault(name, {})[lane + "_ms"] = (time.perf_counter() - t) * 1e3
            t = time.perf_counter()
            tickets = [srv.submit(**reqs["tg3d64_fp64"]) for _ in range(16)]
            for x in tickets:
                srv.wait(x, 600.0)
            out.setdefault("16x_tg3d64_fp64", {})[lane + "_ms"] = (time.perf_counter() - t) * 1e3
    return out


def run_serve(args):
    import numpy as np
    import torch
    import erlbm_gb300 as E
    torch.cuda.set_device(0)
    stream = serve_stream(E, args.requests, args.rate)

    def serve(team_ctas, clocked):
        """The stream through one server: (results, clock record)."""
        with E.Server(hbm_budget_bytes=16 << 30, team_ctas=team_ctas, team_max_nodes=args.team_max_nodes) as srv:
            # warm-up: one request of each kind
            for _, r in stream[:8]:
                srv.wait(srv.submit(**dict(r, n_steps=min(r["n_steps"], 10))))
            clocks = Clocks(0)
            if clocked:
                clocks.start()
            t0 = time.perf_counter()
            tickets = []
            for at, r in stream:
                now = time.perf_counter() - t0
                if at > now:
                    time.sleep(at - now)
                tickets.append(srv.submit(**r))
            res = [srv.wait(t, 3600.0) for t in tickets]
            clk = clocks.stop() if clocked else None
        ok = [x for x in res if x["status"] == 0]
        lat = np.array([x["t_done"] - x["t_submit"] for x in ok])
        span = max(x["t_done"] for x in ok) - min(x["t_submit"] for x in ok)
        return res, ok, lat, span, clk

    res, ok, lat, span, clk = serve(args.team_ctas, True)
    value = len(ok) / span
    singles = serve_single_runs(E, args) if args.single_runs else None
    stream_only = None
    if not args.no_extras and args.team_ctas >= 0:
        # the same stream with every non-slot request on the host-launched stream lane
        _, ok2, lat2, span2, _ = serve(-1, False)
        stream_only = {"value": len(ok2) / span2, "unit": "runs/s", "p50": float(np.percentile(lat2, 50)),
                       "p99": float(np.percentile(lat2, 99)), "failed": args.requests - len(ok2)}
    # the plain path on an evenly strided sample of the same stream, one run after another
    m = max(1, min(args.plain_requests, len(stream)))
    sample = stream[:: max(1, len(stream) // m)][:m]
    t = time.perf_counter()
    for _, r in sample:
        plain_run(E, r)
    plain = len(sample) / (time.perf_counter() - t)
    line = {"metric": "served runs/s", "value": value, "unit": "runs/s", "n_gpus": 1, "steps": len(ok),
            "warmup": 8, "ms_per_step": span / max(1, len(ok)) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded Poisson stream of config-5 requests)",
            "config": {"workload": f"serve {args.requests} requests, Poisson {args.rate:.0f}/s, mixed kinds",
                       "requests": args.requests, "team_ctas": args.team_ctas,
                       "team_max_nodes": args.team_max_nodes},
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "max": float(lat.max())},
            "failed": len(res) - len(ok), "lanes": {"resident": sum(1 for x in ok if x["lane"] == 0),
                                                    "team": sum(1 for x in ok if x["lane"] == 2),
                                                    "stream": sum(1 for x in ok if x["lane"] == 1)},
            "plain_fp64_one_run_at_a_time": {"value": plain, "unit": "runs/s", "requests": len(sample),
                                             "sample": "every k-th request of the same stream"},
            "stream_lane_only": stream_only,
            "single_runs": singles,
            "roofline": None, "e2e": {"value": value, "unit": "runs/s", "h2d_bytes_per_step": 64,
                                      "d2h_bytes_per_step": 64},
            "gpu_launches": None, "clocks": clk}
    print(json.dumps(line), flush=True)
    return 0


def run_snapshot(args):
    """Snapshots of the double shear layer as the program writes them at each interval: the kinetic
    energy and the ASCII velocity and vorticity files (rec_velocity, rec_vorticity), wall-clock per
    snapshot, the files written to a scratch directory and removed after each timed snapshot."""
    import shutil
    import tempfile
    import numpy as np
    import torch
    import erlbm_gb300 as E
    torch.cuda.set_device(0)
    L = args.L
    prec = E.FP64 if args.precision == "fp64" else E.FP32_SHIFTED
    op, tnh, op_label = DSL_OPS[args.op]
    lat = E.Lattice(9, L, L, 1, None, tau_of(L), tnh, op, prec)
    lat.set_populations(E.init_double_shear(L))
    lat.step(101)
    lat.sync()
    d = tempfile.mkdtemp(prefix="erlbm_snap_")

    def snap(fmt):
        t = time.perf_counter()
        lat.kinetic_energy(E.STAGE_POST_COLLISION)
        lat.write_vtk(os.path.join(d, "vel.vtk"), E.FIELD_VELOCITY, fmt)
        lat.write_vtk(os.path.join(d, "vor.vtk"), E.FIELD_VORTICITY, fmt)
        dt = time.perf_counter() - t
        size = os.path.getsize(os.path.join(d, "vel.vtk")) + os.path.getsize(os.path.join(d, "vor.vtk"))
        os.remove(os.path.join(d, "vel.vtk"))
        os.remove(os.path.join(d, "vor.vtk"))
        return dt, size

    try:
        for _ in range(args.warmup):
            snap(E.VTK_ASCII)
        clocks = Clocks(0)
        clocks.start()
        ts = [snap(E.VTK_ASCII) for _ in range(args.steps)]
        clk = clocks.stop()
        tb = [snap(E.VTK_BINARY_FLOAT) for _ in range(max(1, args.steps // 2))]
        cpu = None
        if not args.no_cpu:
            from oracle import oracle as O
            aos = lat.get_populations(E.STAGE_POST_COLLISION)
            ol = O.Lattice(9, L, L, 1, None, tau_of(L), tnh, op)
            ol.set(aos)
            t = time.perf_counter()
            ol.kinetic_energy(0)
            O.write_vtk(9, L, L, 1, None, aos, O.FIELD_VELOCITY, O.VTK_ASCII, os.path.join(d, "vel.vtk"))
            O.write_vtk(9, L, L, 1, None, aos, O.FIELD_VORTICITY, O.VTK_ASCII, os.path.join(d, "vor.vtk"))
            tc = time.perf_counter() - t
            cpu = {"value": 1.0 / tc, "unit": "snapshots/s", "cores": 1, "kind": "port",
                   "sample": f"one snapshot at L={L} from host AoS FP64 populations (energy, ASCII velocity "
                             "and vorticity VTK, one thread as the reference's writers)"}
    finally:
        shutil.rmtree(d, ignore_errors=True)
        lat.close()
    sec = sum(t for t, _ in ts) / len(ts)
    n = L * L
    line = {"metric": "snapshots/s", "value": 1.0 / sec, "unit": "snapshots/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if prec == E.FP32_SHIFTED else "f64",
            "data": "synthetic (double shear layer after 101 steps)",
            "config": {"workload": f"double shear layer snapshot L={L} ({op_label}): kinetic energy + "
                                   "rec_velocity + rec_vorticity ASCII VTK", "L": L,
                       "precision": args.precision},
            "bytes_written_per_snapshot": ts[0][1],
            "binary_float": {"value": len(tb) / sum(t for t, _ in tb), "unit": "snapshots/s",
                             "bytes_written_per_snapshot": tb[0][1]},
            "roofline": None,
            "e2e": {"value": 1.0 / sec, "unit": "snapshots/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 8 + 2 * 3 * n * 8},
            "gpu_launches": None, "clocks": clk}
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line))
    return 0


def channel_geometry(ny: int):
    """Solid mask of the channel workload: x and y walls, a cylinder of radius ny / 12 at (ny, ny / 2)."""
    import numpy as np
    nx = 4 * ny
    s = np.zeros((ny, nx), np.uint8)
    s[:, 0] = s[:, nx - 1] = 1
    s[0, :] = s[ny - 1, :] = 1
    yy, xx = np.mgrid[0:ny, 0:nx]
    s[(xx - ny) ** 2 + (yy - ny // 2) ** 2 <= (ny // 12) ** 2] = 1
    return nx, s.reshape(-1)


def run_channel(args):
    import numpy as np
    import torch
    import erlbm_gb300 as E
    torch.cuda.set_device(0)
    ny = max(64, args.L // 2)
    nx, solid = channel_geometry(ny)
    prec = E.FP64 if args.precision == "fp64" else E.FP32_SHIFTED
    tau, tnh, op = 0.55, 0.7, E.OP_EXTREG
    bc = dict(inlet_x=1, inlet_kind=E.INLET_PARABOLIC, parabolic_L=ny - 2, u_in=0.05, outlet_x=nx - 2,
              outlet_kind=E.OUTLET_CONVECTIVE)
    lat = E.Lattice(9, nx, ny, 1, solid, tau, tnh, op, prec)
    n_fluid = lat.n_fluid
    f0 = np.tile(np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4), n_fluid)
    stream = torch.cuda.Stream()
    lat.set_stream(stream.cuda_stream)
    lat.set_populations(f0)
    inner, K, W = args.inner, args.steps, args.warmup
    for _ in range(W):
        lat.step(inner, bc)
    lat.sync()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(K):
        lat.step(inner, bc)
    ev1.record(stream)
    stream.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    value = n_fluid * inner * K / (ms / 1e3) / 1e6
    launch_ms = ms / (K * inner)
    bpl = BYTES_PER_LU["fp64" if prec == E.FP64 else "fp32"]
    peak, peak_kind = peaks()
    achieved = bpl * n_fluid / (launch_ms / 1e3) / 1e9
    # end to end through the C ABI: populations from pinned host memory, inner steps, energy back
    pinned = torch.empty(f0.size, dtype=torch.float64, pin_memory=True)
    pinned.numpy()[:] = f0
    host = pinned.numpy()
    lat.set_populations(host)
    lat.step(inner, bc)
    lat.kinetic_energy(E.STAGE_POST_COLLISION)
    t0 = time.perf_counter()
    for _ in range(K):
        lat.set_populations(host)
        lat.step(inner, bc)
        lat.kinetic_energy(E.STAGE_POST_COLLISION)
    t_e2e = time.perf_counter() - t0
    lat.close()
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        ol = O.Lattice(9, nx, ny, 1, solid, tau, tnh, op)
        ol.set(f0)
        ol.step(10, bc, threads=threads)
        n_cpu = 10
        t = time.perf_counter()
        while True:
            ol.step(n_cpu, bc, threads=threads)
            dt = time.perf_counter() - t
            if dt > 0.5 or n_cpu > 100000:
                break
            t = time.perf_counter()
            n_cpu *= 4
        cpu = {"value": n_fluid * n_cpu / dt / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
               "sample": f"the same channel, FP64, {n_cpu} steps, {threads} OpenMP threads"}
    line = {"metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": 1, "steps": K, "warmup": W,
            "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == E.FP64 else "f32", "data": "synthetic (channel at rest, parabolic inflow)",
            "config": {"workload": f"D2Q9 channel {nx}x{ny} with a cylinder, parabolic inlet, convective outlet, "
                                   f"E-RLBM tau=0.55 tau_nh=0.7", "nx": nx, "ny": ny, "n_fluid": n_fluid,
                       "lbm_steps_per_step": inner, "precision": args.precision,
                       "l2": f"working set {bpl * n_fluid / 1e6:.0f} MB (two population buffers) "
                             f"{'>' if bpl * n_fluid > 129e6 else '<'} 129 MB L2, no flush"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "traffic": channel_traffic(nx, ny) if prec != E.FP64 else None,
                         "algorithmic_bytes_per_launch": bpl * n_fluid,
                         "launch_us": launch_ms * 1e3, "lattice_updates_per_launch": n_fluid,
                         "kernel": "k_step<PrecExact64,9,4>" if prec == E.FP64 else "k_d2q9_hybrid<4>"},
            "e2e": {"value": n_fluid * inner * K / t_e2e / 1e6, "unit": "MLUPS",
                    "h2d_bytes_per_step": int(f0.nbytes), "d2h_bytes_per_step": 8},
            "gpu_launches": K * inner, "clocks": clk}
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload in ("tg-map", "obstacle-map"):
        return run_map(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "snapshot":
        return run_snapshot(args)
    if args.workload == "channel":
        return run_channel(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
