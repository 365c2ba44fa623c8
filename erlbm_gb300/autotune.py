"""Autotuner for the launch shapes of the hot kernels.

Two shapes are tuned by measurement on the GPU at hand:
  * the fused periodic D2Q9 FP32 kernel: threads per block (128 / 256 / 512), plain or streaming
    (evict-first) stores, and one or two steps per launch, per lattice side L;
  * the persistent map kernel: resident lattices ("slots") per SM, per map kind and precision.
Each candidate is timed with CUDA events after a warm-up; the winner is cached in a JSON file
($ERLBM_TUNE_CACHE, default ~/.cache/erlbm_gb300/autotune.json) keyed by the device name, so later
runs reuse it.  map_run(..., slots=-1) and apply_periodic() read the cache.
"""
from __future__ import annotations

import json
import os
import threading

_lock = threading.Lock()


def cache_path() -> str:
    return os.environ.get("ERLBM_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "erlbm_gb300",
                                                           "autotune.json"))


def _device_key() -> str:
    import torch
    return torch.cuda.get_device_name(torch.cuda.current_device()).replace(" ", "_")


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except Exception:
        return {}


def _store(key: str, value) -> None:
    with _lock:
        d = _load()
        d[key] = value
        os.makedirs(os.path.dirname(cache_path()), exist_ok=True)
        # a file of this process's own, renamed over the cache: ranks of one job that tune at the
        # same time each replace the whole file and never read a half-written one
        tmp = f"{cache_path()}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, cache_path())


def _time_steps(lat, stream, n: int) -> float:
    import torch
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    lat.step(n)
    b.record(stream)
    stream.synchronize()
    return a.elapsed_time(b) / 1e3


PERIODIC_CANDIDATES = [(128, False), (256, False), (512, False), (128, True), (256, True), (512, True)]
# two and three steps per launch: one kernel shape each (warp strips in 128-thread CTAs); the block size
# given with them is the one-step shape used for the steps a call has left over
MULTI_STEP_CANDIDATES = [(128, False, 2), (128, False, 3), (128, True, 3)]  # (block, wide strips, steps)


def tune_periodic(L: int, steps: int = 200, force: bool = False) -> dict:
    """Best (block_threads, streaming_stores, two_step, three_step) of the fused D2Q9 FP32 kernel on an
    L x L lattice."""
    import torch
    import erlbm_gb300 as E
    key = f"{_device_key()}/periodic_d2q9_fp32/shapes4/L{L}"
    hit = _load().get(key)
    if hit and not force:
        return hit
    if L % 128:
        raise ValueError("the fused kernel needs L % 128 == 0")
    stream = torch.cuda.Stream()
    results = []
    with E.Lattice(9, L, L, 1, None, 0.5 + 3.0 * (1 / 32) * L / 80000.0, 0.65, E.OP_EXTREG, E.FP32_SHIFTED) as lat:
        lat.set_stream(stream.cuda_stream)
        lat.set_populations(E.init_double_shear(L))
        lat.step(1)
        cands = [(b, s, False, 1) for b, s in PERIODIC_CANDIDATES]
        if L % 2 == 0 and L >= 4:
            cands += [(b, False, w, per) for b, w, per in MULTI_STEP_CANDIDATES if not w or L >= 16]
        for block, st, wide, per in cands:
            lat.set_launch(block, st, per == 2, per == 3, wide)
            lat.step(20)
            t = min(_time_steps(lat, stream, steps) for _ in range(3))
            results.append(dict(block_threads=block, streaming_stores=st, two_step=per == 2, three_step=per == 3,
                                wide_strips=wide, mlups=L * L * steps / t / 1e6))
    best = max(results, key=lambda r: r["mlups"])
    out = dict(best, candidates=results)
    _store(key, out)
    return out


def apply_periodic(lat) -> dict | None:
    """Sets a lattice's launch shape from the cache (tuning first if the side fits and nothing is cached)."""
    if lat.q != 9 or lat.precision != 1 or lat.nx % 128 or lat.nz != 1:
        return None
    best = tune_periodic(lat.nx)
    lat.set_launch(best["block_threads"], best["streaming_stores"], best.get("two_step", False),
                   best.get("three_step", False), best.get("wide_strips", False))
    return best


def tune_map(kind: int, precision: int, map_points: int = 40, max_steps: int = 3000, force: bool = False) -> dict:
    """Best resident lattices per SM for the persistent map kernel."""
    import time
    import torch
    import erlbm_gb300 as E
    key = f"{_device_key()}/map/{kind}/{precision}"
    hit = _load().get(key)
    if hit and not force:
        return hit
    step = 400 / map_points
    pts = [(int(i * step), int(j * step)) for j in range(map_points) for i in range(map_points)]
    op = 0 if kind == E.MAP_TAYLOR_GREEN else E.OP_EXTREG
    results = []
    for slots in (1, 2, 3, 4):
        try:
            E.map_run(kind, pts[:64], precision=precision, op=op, max_steps=200, slots=slots)
            torch.cuda.synchronize()
            t = time.perf_counter()
            lab, dec, _ = E.map_run(kind, pts, precision=precision, op=op, max_steps=max_steps, slots=slots)
            dt = time.perf_counter() - t
        except E.ErlbmError:
            continue
        results.append(dict(slots=slots, runs_per_s=len(lab) / dt))
    best = max(results, key=lambda r: r["runs_per_s"])
    out = dict(best, candidates=results)
    _store(key, out)
    return out


def best_slots(kind: int, precision: int) -> int:
    """Cached slots per SM for a map kind and precision, 0 (as many as fit) if none is cached."""
    try:
        hit = _load().get(f"{_device_key()}/map/{kind}/{precision}")
    except Exception:
        hit = None
    return int(hit["slots"]) if hit else 0
