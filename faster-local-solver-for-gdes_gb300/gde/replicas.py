"""Replica execution across GPUs: every rank holds the whole graph and solves
its own contiguous shard of the queries; nothing crosses GPUs while pushing.

Queries, seeds and feature columns of these solvers are independent
(each is its own linear system), so the only exchange is collecting the
per-query results on the host afterwards (``torch.distributed`` object
gather over whatever backend the process group uses).  One process per GPU,
as launched by ``torch.distributed.run``.
"""
from __future__ import annotations

from typing import Callable

import numpy as np


def shard_bounds(n_items: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous, balanced [lo, hi) share of ``n_items`` for ``rank`` of ``world``."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of world {world}")
    return n_items * rank // world, n_items * (rank + 1) // world


def _world(group):
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return 1, 0
    return dist.get_world_size(group), dist.get_rank(group)


def solve_sharded(seeds, eps, solve: Callable[..., dict], *, group=None, gather_keys=("oper", "rounds"),
                  **solve_kw) -> dict:
    """Solve this rank's shard of (seeds, eps) with ``solve(seeds, eps, **solve_kw)``.

    ``solve`` returns a dict of per-query arrays (``gde.api.solve`` does).
    Returns ``{"lo", "hi", "local": <this rank's result>, <key>: <all ranks'
    values in query order> for key in gather_keys}``.
    """
    seeds = np.asarray(seeds)
    eps = np.broadcast_to(np.asarray(eps, dtype=np.float64), seeds.shape)
    world, rank = _world(group)
    lo, hi = shard_bounds(seeds.shape[0], world, rank)
    local = solve(seeds[lo:hi], eps[lo:hi], **solve_kw)
    out = {"lo": lo, "hi": hi, "local": local}
    mine = {k: np.asarray(local[k]) for k in gather_keys}
    if world == 1:
        out.update(mine)
        return out
    import torch.distributed as dist
    parts = [None] * world
    dist.all_gather_object(parts, (lo, hi, mine), group=group)
    parts.sort(key=lambda p: p[0])
    for k in gather_keys:
        out[k] = np.concatenate([p[2][k] for p in parts])
    return out
