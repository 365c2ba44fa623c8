"""Sharding of independent runs (stability-map points) across ranks.

Map points are independent (each is its own roda_ponto), so N processes -- one per GPU -- take
disjoint, strided shares of the point list and exchange only their labels at the end; there is no
collective on the data path.  The gather uses torch.distributed (NCCL between GPUs, gloo on CPU).
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np


def shard(points: Sequence, rank: int, world: int) -> list:
    """Strided share of `points` for `rank`: long and short runs interleave, so shares balance."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return list(points[rank::world])


def unshard(parts: Sequence[np.ndarray], n: int, world: int) -> np.ndarray:
    """Inverse of shard(): parts[r] holds the results of points r, r + world, ..."""
    out = None
    for r, p in enumerate(parts):
        p = np.asarray(p)
        if out is None:
            out = np.empty((n,) + p.shape[1:], dtype=p.dtype)
        out[r::world] = p[: len(range(r, n, world))]
    return out


def run_sharded(points: Sequence, runner: Callable[[list], tuple], group=None):
    """Runs `runner` (e.g. a map_run over a point list returning (labels, decided, margins)) on this
    rank's share and gathers every rank's results in the original point order on all ranks.  Each
    result array holds one value per point; its dtype is kept (labels and steps are exact in the
    float64 the gather carries)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    mine = shard(points, rank, world)
    res = runner(mine)
    if world == 1:
        return tuple(np.asarray(r) for r in res)
    n = len(points)
    per = (n + world - 1) // world
    out = []
    for arr in res:
        arr = np.asarray(arr)
        dtype = arr.dtype
        pad = np.zeros(per, dtype=np.float64)
        pad[: arr.size] = arr.astype(np.float64)
        t = torch.from_numpy(pad)
        if dist.get_backend(group) == "nccl":
            t = t.cuda()
        bufs = [torch.zeros_like(t) for _ in range(world)]
        dist.all_gather(bufs, t, group=group)
        parts = [b.cpu().numpy() for b in bufs]
        out.append(unshard(parts, n, world).astype(dtype))
    return tuple(out)


def map_run_sharded(kind: int, points=None, map_fn: Callable | None = None, group=None, **kw):
    """A stability map split over the ranks of a process group: each rank (one GPU) runs its strided
    share of the points with `map_fn` (default erlbm_gb300.map_run, called as map_fn(kind, points, **kw))
    and every rank receives all results in point order, as map_run returns them for the whole list.

    points: (i, j) map indices, or None for the whole n_i x n_j grid (i fastest), as in map_run.  On the
    Taylor-Green map with op = 0 every point runs with RLBM and with E-RLBM, and the results are laid
    out as map_run lays them out: all RLBM results, then all E-RLBM results.  The replacement for the
    maps' OpenMP loop over points (main_stability-map_taylor-green.cpp:150-166,
    main_stability-map_obstacle.cpp:161-175) across GPUs; the only exchange is the gather."""
    if map_fn is None:
        from . import map_run as map_fn
    if points is None:
        n_i, n_j = kw.get("n_i", 400), kw.get("n_j", 400)
        points = [(i, j) for j in range(n_j) for i in range(n_i)]
    points = [tuple(p) for p in points]
    doubled = kind == 1 and kw.get("op", 4) == 0  # MAP_TAYLOR_GREEN with both operators

    def runner(mine):
        lab, dec, mg = map_fn(kind, mine, **kw)
        if not doubled:
            return lab, dec, mg
        m = len(mine)
        return lab[:m], lab[m:], dec[:m], dec[m:], mg[:m], mg[m:]

    res = run_sharded(points, runner, group)
    if not doubled:
        return res
    return tuple(np.concatenate([res[2 * k], res[2 * k + 1]]) for k in range(3))
