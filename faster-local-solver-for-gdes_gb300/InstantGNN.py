"""Drop-in GPU replacement of the reference's ``InstantGNN.py`` (dynamic feature propagation).

Generalised PPR with exponent beta over every feature column:
    p_u += alpha r_u;  r_v += (1-alpha) r_u / d_u^{1-beta} / d_v^beta;  threshold d_u^{1-beta} eps
(InstantGNN.py:12-43).  All F columns are pushed together in node x column
tiles on the GPU; P and R (n x F numpy arrays) are updated in place like the
reference's.  The forward push is synchronous: each round every node whose
residual passes its threshold pushes.  The SOR push (omega != 1,
instantGNNSorPush, InstantGNN.py:74-105) relaxes in multicolour
Gauss-Seidel order: all pending nodes of one colour of a proper colouring
at once.
"""
from __future__ import annotations

import numpy as np

from gde import _lib as L
from gde import api
from gde.dropin import Timer, graph_for

__all__ = ["instantGNNParallel", "instantGNNSorParallel", "instantGNNUpdateBatchParallel"]


def _dev(g):
    return f"cuda:{g.ctx.device}"


def _to_dev(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)


def instantGNNParallel(n, indptr, indices, degree, alpha, eps, P, R, beta, batchsize=80, omega=1.0):
    """Static propagation of every column (InstantGNN.py:46-71) -> runtimes[F]; P, R updated in place."""
    g = graph_for(indptr, indices, degree, padded=True)
    dev = _dev(g)
    Rd = _to_dev(R, dev)
    Pd = _to_dev(np.zeros_like(R), dev)
    with Timer() as t:
        api.feature_push(g, L.IGN, Pd, Rd, eps, alpha=alpha, beta=beta, prec="fp64", omega=omega)
    P[:] = Pd.cpu().numpy()
    R[:] = Rd.cpu().numpy()
    F = R.shape[1]
    return np.full(F, t.dt / max(F, 1))


def instantGNNSorParallel(n, indptr, indices, degree, alpha, eps, omega, P, R, beta, batchsize=80):
    """SOR propagation of every column (InstantGNN.py:108-134), multicolour order -> runtimes[F]."""
    return instantGNNParallel(n, indptr, indices, degree, alpha, eps, P, R, beta, batchsize, omega=omega)


def instantGNNUpdateBatchParallel(n, indptr, indices, degree, alpha, eps, omega, P, R, X, us, vs, beta, algo,
                                  batchsize=80):
    """Snapshot update (InstantGNN.py:332-359): edits indices/degree in place, repairs and pushes P, R.

    ``algo`` containing 'insert' inserts only (updetaGraph onlyinsert=True);
    otherwise edges already present are deleted.
    """
    assert indices.dtype == np.int32 and degree.dtype == np.int64, "indices int32 and degree int64 (as the reference)"
    g = graph_for(indptr, indices, degree, padded=True)
    dev = _dev(g)
    Pd = _to_dev(P, dev)
    Rd = _to_dev(R, dev)
    Xd = _to_dev(X, dev)
    with Timer() as t:
        api.feature_update(g, L.IGN, indices, degree, us, vs, "insert" in algo, Pd, Rd, Xd, eps, alpha=alpha,
                           beta=beta, prec="fp64", omega=omega if "sor" in algo else 1.0)
    # the resident graph now matches the mutated arrays: re-key the cache
    from gde import dropin
    dropin.forget(g)
    key = (dropin._fingerprint(indptr), dropin._fingerprint(indices), dropin._fingerprint(np.asarray(degree)), True)
    dropin._CACHE[key] = g
    P[:] = Pd.cpu().numpy()
    R[:] = Rd.cpu().numpy()
    F = R.shape[1]
    return np.full(F, t.dt / max(F, 1))
