"""Loader for ``tests/golden/golden_reference.npz`` (outputs of the reference itself).

``tests/golden/make_golden.py`` ran the reference's own CPU code on small
seeded graphs and stored, per case, its kind, graph, parameters and outputs.
"""
from __future__ import annotations

import functools
import os

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_reference.npz")


@functools.lru_cache(maxsize=1)
def load() -> dict:
    z = np.load(PATH)
    return {k: z[k] for k in z.files}


def graphs() -> dict:
    d = load()
    out = {}
    for k in d:
        if k.startswith("graph/"):
            _, name, field = k.split("/")
            out.setdefault(name, {})[field] = d[k]
    return out


def cases(kind: str | None = None) -> list[dict]:
    d = load()
    by = {}
    for k, v in d.items():
        if not k.startswith("case"):
            continue
        parts = k.split("/")
        c = by.setdefault(parts[0], {"id": parts[0], "p": {}, "o": {}})
        if parts[1] in ("kind", "graph"):
            c[parts[1]] = str(v)
        else:
            c[parts[1]][parts[2]] = v[()] if v.ndim == 0 else v
    out = [by[k] for k in sorted(by)]
    if kind is not None:
        out = [c for c in out if c["kind"] == kind]
    return out


def dyn() -> dict:
    d = load()
    return {k.split("/", 1)[1]: v for k, v in d.items() if k.startswith("dyn/")}
