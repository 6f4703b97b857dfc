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
from gde.dropin import (Timer, column_repair_push, edit_batch, eps_from_vec, graph_for, neighbour_maps,
                        queue_entries, rekey, repair_lists)

__all__ = ["instantGNNParallel", "instantGNNSorParallel", "instantGNNUpdateBatchParallel", "instantGNNPush",
           "instantGNNSorPush", "updetaGraph", "instantGNNUpdateBatch"]


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
    rekey(g, indptr, indices, degree)  # the resident graph already holds the edit
    P[:] = Pd.cpu().numpy()
    R[:] = Rd.cpu().numpy()
    F = R.shape[1]
    return np.full(F, t.dt / max(F, 1))


def _column(g, a):
    import torch
    return torch.from_numpy(np.asarray(a, dtype=np.float64).reshape(-1, 1).copy()).to(_dev(g))


def _push_column(n, indptr, indices, degree, alpha, eps_vec, p, r, queue, front, rear, q_mark, beta, omega):
    g = graph_for(indptr, indices, degree, padded=True)
    eps = eps_from_vec(eps_vec, np.power(np.asarray(degree, dtype=np.float64), 1 - beta))
    cand = np.unique(queue_entries(queue, front, rear, n))
    P, R = _column(g, p), _column(g, r)
    with Timer() as t:
        if cand.size:
            api.feature_push(g, L.IGN, P, R, eps, alpha=alpha, beta=beta, prec="fp64", cand=cand, tile_w=1,
                             omega=omega)
    p[:] = P[:, 0].cpu().numpy()
    r[:] = R[:, 0].cpu().numpy()
    q_mark[:] = False
    return t.dt


def instantGNNPush(n, indptr, indices, degree, alpha, eps_vec, p, r, queue, front, rear, q_mark, beta):
    """Push one feature column from the nodes in its queue (InstantGNN.py:12-43) on the device -> runtime.

    ``n`` is the queue's length (the reference passes the node count + 2),
    the queue holds entries front+1 .. rear; eps_vec must be
    degree^(1-beta) * eps.  p, r are updated in place.  The push is
    synchronous: every node at or above its threshold pushes each round.
    """
    return _push_column(n, indptr, indices, degree, alpha, eps_vec, p, r, queue, front, rear, q_mark, beta, 1.0)


def instantGNNSorPush(n, indptr, indices, degree, alpha, eps_vec, omega, p, r, queue, front, rear, q_mark, beta):
    """Relaxed push of one feature column (InstantGNN.py:74-105) in multicolour SOR order -> runtime."""
    return _push_column(n, indptr, indices, degree, alpha, eps_vec, p, r, queue, front, rear, q_mark, beta, omega)


def updetaGraph(indptr, indices, degree, us, vs, onlyinsert=True):
    """Edge batch on the padded CSR (InstantGNN.py:137-180), on the device; indices / degree edited in place
    -> (insert_neighbor, delete_neighbor): node -> neighbours inserted / deleted, in batch order."""
    _, outcome = edit_batch(indptr, indices, degree, us, vs, onlyinsert)
    return neighbour_maps(np.asarray(us), np.asarray(vs), outcome)


def instantGNNUpdateBatch(n, indptr, indices, degree, old_degree, p, r, x, alpha, queue, front, rear, q_mark, eps_vec,
                          insert_neighbor, delete_neighbor, algo='fwd', omega=1, beta=0):
    """One feature column after updetaGraph (InstantGNN.py:298-329) on the device: repair p, r at the nodes
    with insertions (deleted neighbours count unless ``algo`` contains 'insert'), then push from them ('sor':
    multicolour SOR with omega, 'fwd': synchronous).  p, r updated in place -> runtime."""
    g = graph_for(indptr, indices, degree, padded=True)
    eps = eps_from_vec(eps_vec, np.power(np.asarray(degree, dtype=np.float64), 1 - beta))
    keys, old_deg, off, nbr = repair_lists(insert_neighbor, delete_neighbor, old_degree,
                                                       'insert' not in algo)
    pending = queue_entries(queue, front, rear, n + 2)
    push = omega if 'sor' in algo else (1.0 if 'fwd' in algo else None)
    with Timer() as t:
        column_repair_push(g, L.IGN, p, r, x, keys, old_deg, off, nbr, pending, alpha, eps, beta, push)
    q_mark[:] = False
    return t.dt

