"""Autotuner for batched solves: tile width, serving slots and degree buckets.

Times ``api.solve`` on a sample of the caller's queries for each candidate
configuration (device time of the call, best of ``reps``) and keeps the
fastest, or, with ``max_p99_ms``, the fastest whose 99th-percentile query
latency (device time from a query's start to its finish) stays within the
bound.  The search is staged: first the execution shape (served slots
for single-column tiles, or node x column tiles of width 4..32), then the
degree-bucket thresholds (rows per lane / per warp, long-row chunk) for the
winning shape, and for served shapes the number of block groups the slots
share.  Results are cached per graph, kind, precision, sample size
and latency bound in a JSON file next to the graph cache, so a workload is
tuned once.
"""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

from gde import _lib as L
from gde import api

SHAPES = [
    {"tile_w": 1, "slots": 32},
    {"tile_w": 1, "slots": 64},
    {"tile_w": 1, "slots": 128},
    {"tile_w": 1, "slots": 256},
    {"tile_w": 4},
    {"tile_w": 8},
    {"tile_w": 16},
    {"tile_w": 32},
]
BUCKETS = [
    {},
    {"small_max": 16},
    {"small_max": 4},
    {"med_max": 1024, "chunk": 1024},
    {"med_max": 128, "chunk": 128},
]
# served shapes: slots per block group (the engine's default is one group per
# slot for PPR queues, one per 8 slots with Katz or heat-kernel queries)
SLOTS_PER_GROUP = [2, 8]


def _cache_path(graph: api.Graph, key: str) -> str:
    d = os.environ.get("GDE_GRAPH_CACHE") or os.path.join(
        os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), ".graph_cache")
    os.makedirs(os.path.join(d, "tune"), exist_ok=True)
    return os.path.join(d, "tune", key + ".json")


def _graph_key(graph: api.Graph, kind: int, prec: str, n_sample: int, max_p99_ms) -> str:
    h = hashlib.sha1(f"{graph.n}:{graph.cap}:{graph.vol}:{kind}:{prec}:{n_sample}:{max_p99_ms}".encode())
    return f"g{graph.n}_{h.hexdigest()[:16]}"


def _time(graph, kind, seeds, eps, prec, alpha, cfg, reps) -> tuple[float, float]:
    """(best total ms, p99 query latency ms of that run)."""
    tuning = {k: v for k, v in cfg.items() if k != "tile_w"}
    best, p99 = float("inf"), float("inf")
    for _ in range(reps):
        r = api.solve(graph, kind, L.LOCAL_GD, seeds, eps, prec=prec, alpha=alpha, tile_w=cfg["tile_w"],
                      want_x=False, want_r=False, tuning=tuning)
        if r["stats"]["total_ms"] < best:
            best = r["stats"]["total_ms"]
            p99 = float(np.percentile(r["latency_ms"], 99))
    return best, p99


def _pick(table, max_p99_ms):
    ok = [t for t in table if max_p99_ms is None or t[2] <= max_p99_ms]
    return min(ok or table, key=lambda t: t[1] if ok else t[2])


def autotune(graph: api.Graph, kind: int, seeds, eps, *, prec: str = "fp32", alpha: float = 0.1, reps: int = 2,
             shapes=None, buckets=None, slots_per_group=None, use_cache: bool = True,
             max_p99_ms: float | None = None) -> dict:
    """Best configuration for solving queries like (seeds, eps) on ``graph``.

    ``max_p99_ms``: keep only configurations whose p99 query latency is
    within it (the one with the lowest p99 if none is).  Returns
    ``{"tile_w": W, "tuning": {...}, "ms": t, "p99_ms": l, "table": [(cfg, ms, p99), ...]}``;
    pass ``tile_w`` and ``tuning`` to ``api.solve``.
    """
    seeds = np.ascontiguousarray(seeds, dtype=np.int32)
    eps = np.ascontiguousarray(np.broadcast_to(np.asarray(eps, np.float64), seeds.shape))
    path = _cache_path(graph, _graph_key(graph, kind, prec, seeds.shape[0], max_p99_ms))
    if use_cache and os.path.exists(path):
        with open(path) as fh:
            return json.load(fh)
    table = []
    _time(graph, kind, seeds[:8], eps[:8], prec, alpha, {"tile_w": 1}, 1)  # warm-up
    for cfg in (shapes or SHAPES):
        table.append((dict(cfg), *_time(graph, kind, seeds, eps, prec, alpha, cfg, reps)))
    shape = _pick(table, max_p99_ms)[0]
    for b in (buckets or BUCKETS)[1:]:
        cfg = dict(shape)
        cfg.update(b)
        table.append((cfg, *_time(graph, kind, seeds, eps, prec, alpha, cfg, reps)))
    best = _pick(table, max_p99_ms)[0]
    if best.get("tile_w") == 1 and "slots" in best:
        for spg in (SLOTS_PER_GROUP if slots_per_group is None else slots_per_group):
            cfg = dict(best)
            cfg["groups"] = max(1, cfg["slots"] // spg)
            table.append((cfg, *_time(graph, kind, seeds, eps, prec, alpha, cfg, reps)))
    best, ms, p99 = _pick(table, max_p99_ms)
    out = {"tile_w": best["tile_w"], "tuning": {k: v for k, v in best.items() if k != "tile_w"}, "ms": ms,
           "p99_ms": p99, "max_p99_ms": max_p99_ms, "queries": int(seeds.shape[0]), "table": table}
    if use_cache:
        tmp = path + f".{os.getpid()}.tmp"
        with open(tmp, "w") as fh:
            json.dump(out, fh)
        os.replace(tmp, path)
    return out
