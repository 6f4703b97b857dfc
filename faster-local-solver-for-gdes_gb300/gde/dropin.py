"""Shared plumbing of the drop-in modules: graph residency for numpy callers.

The reference's functions take numpy CSR arrays on every call and its GPU
path uploads them each time (``ppr_solver.py:103-105``).  Here a graph is
uploaded once and reused while the caller passes the same arrays with the
same contents (checked by a fingerprint of sampled entries and sizes).
"""
from __future__ import annotations

import time

import numpy as np

from . import api

_CACHE: dict = {}
_MAX = 4


def _fingerprint(a: np.ndarray) -> tuple:
    a = np.asarray(a)
    if a.size == 0:
        return (0,)
    step = max(1, a.size // 4096)
    s = a.ravel()[::step]
    return (a.shape, str(a.dtype), a.ctypes.data, int(np.asarray(s, dtype=np.float64).sum() * 1000003 % (1 << 61)),
            float(a.ravel()[0]), float(a.ravel()[-1]))


def graph_for(indptr, indices, degree=None, padded: bool = False) -> api.Graph:
    """Resident graph for these numpy arrays (uploaded on first use or on change)."""
    deg = None if degree is None else np.asarray(degree)
    key = (_fingerprint(indptr), _fingerprint(indices), None if deg is None else _fingerprint(deg), padded)
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


def oper_like(degree, value: float):
    """The reference's oper has the dtype of sum(degree): int for integer degrees."""
    if degree is not None and np.issubdtype(np.asarray(degree).dtype, np.integer):
        return int(round(value))
    return float(value)


class Timer:
    def __enter__(self):
        self.t0 = time.perf_counter()
        return self

    def __exit__(self, *exc):
        self.dt = time.perf_counter() - self.t0
