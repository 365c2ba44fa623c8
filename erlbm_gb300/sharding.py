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
    rank's share and gathers every rank's results in the original point order on all ranks."""
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
        arr = np.asarray(arr, dtype=np.float64)
        pad = np.zeros(per, dtype=np.float64)
        pad[: arr.size] = arr
        t = torch.from_numpy(pad)
        if dist.get_backend(group) == "nccl":
            t = t.cuda()
        bufs = [torch.zeros_like(t) for _ in range(world)]
        dist.all_gather(bufs, t, group=group)
        parts = [b.cpu().numpy() for b in bufs]
        out.append(unshard(parts, n, world))
    return tuple(out)
