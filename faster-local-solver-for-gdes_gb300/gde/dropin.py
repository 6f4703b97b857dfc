"""Shared plumbing of the drop-in modules: graph residency for numpy callers.

The reference's functions take numpy CSR arrays on every call and its GPU
path uploads them each time (``ppr_solver.py:103-105``).  Here a graph is
uploaded once and reused while the caller passes arrays with the same
contents.  The key is a CRC-32 of every byte of ``indptr``, ``indices`` and
``degree`` (plus shapes and dtypes), so an in-place edit of any entry is
seen and the graph is uploaded again; functions that edit the arrays
through the library (``updeta_graph``, ``updetaGraph``, the dynamic
updates) re-key the resident graph instead, since its device copy already
holds the edit.
"""
from __future__ import annotations

import time
import zlib

import numpy as np

from . import api

_CACHE: dict = {}
_MAX = 4


def _fingerprint(a) -> tuple:
    a = np.ascontiguousarray(a)
    return (a.shape, str(a.dtype), zlib.crc32(memoryview(a).cast("B")) if a.size else 0)


def _key(indptr, indices, degree, padded: bool) -> tuple:
    return (_fingerprint(indptr), _fingerprint(indices), None if degree is None else _fingerprint(degree), padded)


def graph_for(indptr, indices, degree=None, padded: bool = False) -> api.Graph:
    """Resident graph for these numpy arrays (uploaded on first use or when their contents change)."""
    deg = None if degree is None else np.asarray(degree)
    key = _key(indptr, indices, deg, padded)
    g = _CACHE.get(key)
    if g is not None:
        return g
    if len(_CACHE) >= _MAX:
        _CACHE.pop(next(iter(_CACHE)))
    if padded:
        g = api.Graph(indptr, indices, row_len=np.asarray(degree, dtype=np.int64),
                      degree=np.asarray(degree, dtype=np.float64))
    else:
        g = api.Graph(indptr, indices, degree=None if deg is None else deg.astype(np.float64))
    _CACHE[key] = g
    return g


def forget(g: api.Graph) -> None:
    for k, v in list(_CACHE.items()):
        if v is g:
            del _CACHE[k]


def rekey(g: api.Graph, indptr, indices, degree, padded: bool = True) -> None:
    """The caller's arrays were edited through the library: ``g`` (already edited on the device) is their graph."""
    forget(g)
    _CACHE[_key(indptr, indices, None if degree is None else np.asarray(degree), padded)] = g


def oper_like(degree, value: float):
    """The reference's oper has the dtype of sum(degree): int for integer degrees."""
    if degree is not None and np.issubdtype(np.asarray(degree).dtype, np.integer):
        return int(round(value))
    return float(value)


def eps_from_vec(eps_vec, scale) -> float:
    """The scalar eps behind a threshold vector eps_vec = scale * eps (checked on every node)."""
    eps_vec = np.asarray(eps_vec, dtype=np.float64)
    scale = np.asarray(scale, dtype=np.float64)
    nz = np.flatnonzero(scale > 0)
    if nz.size == 0:
        raise ValueError("eps_vec: no node with a positive threshold scale")
    eps = float(eps_vec[nz[0]] / scale[nz[0]])
    if not np.allclose(eps_vec, scale * eps, rtol=1e-12, atol=0.0):
        raise ValueError("eps_vec is not a scalar eps times the reference's threshold scale")
    return eps


def queue_entries(queue, front: int, rear: int, mod: int) -> np.ndarray:
    """Nodes waiting in a reference ring queue (entries front+1 .. rear, modulo mod)."""
    queue = np.asarray(queue)
    cnt = (int(rear) - int(front)) % int(mod)
    idx = (int(front) + 1 + np.arange(cnt)) % int(mod)
    return queue[idx].astype(np.int32)


def neighbour_maps(us, vs, outcome):
    """insert_neighbor / delete_neighbor in batch order from per-edge outcomes (1 inserted, 2 deleted)."""
    ins, dele = {}, {}
    for e in np.flatnonzero(outcome):
        u, v = int(us[e]), int(vs[e])
        d = ins if outcome[e] == 1 else dele
        d.setdefault(u, []).append(v)
        d.setdefault(v, []).append(u)
    return ins, dele


def edit_batch(indptr, indices, degree, us, vs, onlyinsert):
    assert indices.dtype == np.int32 and degree.dtype == np.int64, "indices int32 and degree int64 (as the reference)"
    g = graph_for(indptr, indices, degree, padded=True)
    res = api.graph_update(g, indices, degree, us, vs, bool(onlyinsert))
    rekey(g, indptr, indices, degree)  # the resident graph already holds the edit
    return g, res["outcome"]


def repair_lists(insert_neighbor, delete_neighbor, old_degree, use_deleted):
    keys = np.fromiter(insert_neighbor.keys(), dtype=np.int32, count=len(insert_neighbor))
    off = [0]
    nbr = []
    for u in keys:
        nbr += insert_neighbor[int(u)]
        off.append(len(nbr))
        if use_deleted:
            nbr += delete_neighbor.get(int(u), [])
        off.append(len(nbr))
    return keys, np.asarray(old_degree)[keys].astype(np.int64), np.asarray(off, np.int64), np.asarray(nbr, np.int32)


def column_repair_push(g, kind, p, r, x, keys, old_deg, off, nbr, pending, alpha, eps, beta, omega):
    """Repair then push one feature column (device copies of p, r written back in place)."""
    import torch
    dev = f"cuda:{g.ctx.device}"
    P = torch.from_numpy(np.asarray(p, dtype=np.float64).reshape(-1, 1).copy()).to(dev)
    R = torch.from_numpy(np.asarray(r, dtype=np.float64).reshape(-1, 1).copy()).to(dev)
    X = None if x is None else torch.from_numpy(np.asarray(x, dtype=np.float64).reshape(-1, 1).copy()).to(dev)
    api.feature_repair(g, kind, P, R, X, keys, old_deg, off, nbr, alpha=alpha, beta=beta)
    cand = np.unique(np.concatenate([keys, pending]).astype(np.int32))
    oper = 0.0
    if cand.size and omega is not None:
        res = api.feature_push(g, kind, P, R, eps, alpha=alpha, beta=beta, prec="fp64", cand=cand, tile_w=1,
                               omega=omega)
        oper = float(res["oper"][0])
    p[:] = P[:, 0].cpu().numpy()
    r[:] = R[:, 0].cpu().numpy()
    return oper


class Timer:
    def __enter__(self):
        self.t0 = time.perf_counter()
        return self

    def __exit__(self, *exc):
        self.dt = time.perf_counter() - self.t0
