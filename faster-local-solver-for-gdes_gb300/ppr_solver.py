"""Drop-in GPU replacement of the reference's ``ppr_solver.py`` (personalized PageRank).

    Q x = b,  Q = I - (1-alpha) A D^{-1},  b = alpha e_s   (ppr_solver.py:18-23)

Same function names, positional arguments and return tuples as the
reference; every solve runs in ``libgde.so`` on the GPU (synchronous local
push, ``csrc/push_engine.cu``).  FP64 functions return float64 arrays;
the ``*_gpu`` functions compute in FP32 residuals with a Kahan-compensated
FP32 solution, like the reference's CuPy path returns float32.

The ``solve_a_graph_*`` drivers and ``init_a_graph`` solve all their seeds
in one batched call per method (the reference runs one numba thread per
seed); each seed's ``algo_time`` is the batched call's wall time divided by
the number of seeds.
"""
from __future__ import annotations

import numpy as np

from gde import _lib as L
from gde import api
from gde.dropin import (Timer, column_repair_push, edit_batch, eps_from_vec, graph_for, neighbour_maps,
                        oper_like, queue_entries, rekey, repair_lists)

__all__ = ["ppr_gd", "ppr_gd_local_gpu", "ppr_gd_standard_gpu", "ppr_cheby", "ppr_sor", "ppr_gd_torch",
           "solve_a_graph_gpu", "solve_a_graph_cheby", "solve_a_graph_torch", "solve_a_graph_all",
           "solve_a_graph_omega", "init_a_graph", "updeta_graph", "update_ppr", "update_ppr_parallel",
           "optimal_omega"]


def _solve1(n, indptr, indices, degree, s_node, alpha, eps, method, prec):
    g = graph_for(indptr, indices, degree)
    assert g.n == n, "n must equal len(indptr) - 1"
    r = api.solve(g, L.PPR, method, [s_node], [eps], prec=prec, alpha=alpha)
    return r["x"][0], r["r"][0], r["oper"][0]


def _seeds(s_nodes) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(s_nodes).ravel(), dtype=np.int32)


def _per_seed(dt: float, k: int) -> np.ndarray:
    return np.full(k, dt / max(k, 1))


def _int_opers(oper) -> np.ndarray:
    return np.rint(np.asarray(oper, dtype=np.float64)).astype(np.int64)


def _batch_gd(n, indptr, indices, degree, alpha, eps, s_nodes, local, prec="fp64"):
    """(opers, per-seed times) of ppr_gd over s_nodes in one batched solve."""
    g = graph_for(indptr, indices, degree)
    assert g.n == n, "n must equal len(indptr) - 1"
    seeds = _seeds(s_nodes)
    assert np.all(eps * np.asarray(degree)[seeds] <= 1.)  # ppr_solver.py:213
    with Timer() as t:
        r = api.solve(g, L.PPR, L.LOCAL_GD if local else L.GLOBAL_GD, seeds, eps, prec=prec, alpha=alpha,
                      want_x=False, want_r=False)
    return r["oper"], _per_seed(t.dt, len(seeds))


def _batch_sor(n, indptr, indices, degree, alpha, eps, omega, s_nodes, local, want_x=False):
    g = graph_for(indptr, indices, degree)
    assert g.n == n, "n must equal len(indptr) - 1"
    seeds = _seeds(s_nodes)
    assert np.all(eps * np.asarray(degree)[seeds] <= 1.)  # ppr_solver.py:340
    with Timer() as t:
        r = api.sor(g, L.PPR, seeds, eps, omega=omega, local=local, alpha=alpha, prec="fp64", want_x=want_x,
                    want_r=want_x)
    return r, _per_seed(t.dt, len(seeds))


def ppr_gd(n, indptr, indices, degree, s_node, alpha, eps, local, opt_x=None, debug=False):
    """Local/global gradient descent for Qx = alpha e_s (ppr_solver.py:208-328) -> (xt, rt, oper, algo_time)."""
    assert eps * degree[s_node] <= 1.
    with Timer() as t:
        x, r, oper = _solve1(n, indptr, indices, degree, s_node, alpha, eps, L.LOCAL_GD if local else L.GLOBAL_GD,
                             "fp64")
    return x, r, oper_like(degree, oper), t.dt


def ppr_gd_local_gpu(n, indptr, indices, degree, s_node, alpha, eps):
    """LocalGD on the GPU, FP32 (ppr_solver.py:82-146) -> (xt, rt, oper, algo_time)."""
    with Timer() as t:
        x, r, oper = _solve1(n, indptr, indices, degree, s_node, alpha, eps, L.LOCAL_GD, "fp32")
    return x, r, float(oper), t.dt


def ppr_gd_standard_gpu(n, indptr, indices, degree, s_node, alpha, eps):
    """Global GD on the GPU, FP32 (ppr_solver.py:26-79) -> (xt, rt, oper, algo_time)."""
    with Timer() as t:
        x, r, oper = _solve1(n, indptr, indices, degree, s_node, alpha, eps, L.GLOBAL_GD, "fp32")
    return x, r, float(oper), t.dt


def ppr_cheby(n, indptr, indices, degree, s_node, alpha, eps, local):
    """Local/global Chebyshev (ppr_solver.py:582-661) -> (xt, rt, oper, algo_time).

    The local variant advances all active nodes synchronously; its next
    frontier is every node whose residual passes eps*alpha*d after the round.
    """
    with Timer() as t:
        x, r, oper = _solve1(n, indptr, indices, degree, s_node, alpha, eps,
                             L.LOCAL_CHEBY if local else L.GLOBAL_CHEBY, "fp64")
    return x, r, oper_like(degree, oper), t.dt


def ppr_sor(n, indptr, indices, degree, s_node, alpha, eps, omega, local, opt_x=None, debug=False):
    """LocalSOR / global SOR (ppr_solver.py:331-461) -> (xt, rt, oper, algo_time).

    Same relaxation and stopping rule as the reference; the GPU relaxes in
    multicolour Gauss-Seidel order (all pending nodes of one colour at once)
    instead of the reference's FIFO queue, so ``oper`` is that order's count.
    """
    assert eps * degree[s_node] <= 1.
    g = graph_for(indptr, indices, degree)
    assert g.n == n, "n must equal len(indptr) - 1"
    with Timer() as t:
        r = api.sor(g, L.PPR, [s_node], [eps], omega=omega, local=local, alpha=alpha, prec="fp64")
    return r["x"][0], r["r"][0], oper_like(degree, r["oper"][0]), t.dt


def ppr_gd_torch(adj_mat, n, degree, deg_mat, alpha, eps, s_node, device):
    """Global GD reference solve (ppr_solver.py:167-188) -> (xt[n,1], rt[n,1], algo_time)."""
    crow = adj_mat.crow_indices().cpu().numpy()
    col = adj_mat.col_indices().cpu().numpy()
    deg = np.asarray(degree.cpu().numpy() if hasattr(degree, "cpu") else degree)
    with Timer() as t:
        x, r, _ = _solve1(n, crow, col, deg, s_node, alpha, eps, L.GLOBAL_GD, "fp64")
    return x.reshape(n, 1), r.reshape(n, 1), t.dt


def solve_a_graph_torch(n, indptr, indices, degree, alpha, eps, s_nodes, device):
    """Mean per-seed time of the global reference solve over s_nodes (ppr_solver.py:191-205)."""
    _, t = _batch_gd(n, indptr, indices, degree, alpha, eps, s_nodes, False)
    return float(np.mean(t))


def solve_a_graph_gpu(n, indptr, indices, degree, alpha, eps, s_nodes):
    """GPU global then local GD over s_nodes, FP32 (ppr_solver.py:149-164) -> (s_nodes, local_times, global_times)."""
    _, gt = _batch_gd(n, indptr, indices, degree, alpha, eps, s_nodes, False, prec="fp32")
    _, lt = _batch_gd(n, indptr, indices, degree, alpha, eps, s_nodes, True, prec="fp32")
    return s_nodes, lt, gt


def solve_a_graph_cheby(n, indptr, indices, degree, alpha, eps, omega, graph_name, s_nodes):
    """Local and global Chebyshev over s_nodes (ppr_solver.py:664-693)
    -> (s_nodes, local_opers, local_times, global_opers, global_times)."""
    g = graph_for(indptr, indices, degree)
    assert g.n == n, "n must equal len(indptr) - 1"
    seeds = _seeds(s_nodes)
    out = []
    for method in (L.LOCAL_CHEBY, L.GLOBAL_CHEBY):
        with Timer() as t:
            r = api.solve(g, L.PPR, method, seeds, eps, prec="fp64", alpha=alpha, want_x=False, want_r=False)
        out += [_int_opers(r["oper"]), _per_seed(t.dt, len(seeds))]
    return (s_nodes, *out)


def solve_a_graph_all(n, indptr, indices, degree, alpha, eps, omega, graph_name, s_nodes):
    """Every PPR method over s_nodes (ppr_solver.py:511-579): local / global SOR with omega, local / global
    APPR (omega = 1), local / global GD -> (s_nodes, local_sor_opers, local_sor_algo_times, global_sor_opers,
    global_sor_algo_times, local_appr_opers, local_appr_algo_times, global_appr_opers, global_appr_algo_times,
    local_gd_opers, local_gd_algo_times, global_gd_opers, global_gd_algo_times)."""
    go, gt = _batch_gd(n, indptr, indices, degree, alpha, eps, s_nodes, False)
    ls, lst = _batch_sor(n, indptr, indices, degree, alpha, eps, omega, s_nodes, True)
    gs, gst = _batch_sor(n, indptr, indices, degree, alpha, eps, omega, s_nodes, False)
    la, lat = _batch_sor(n, indptr, indices, degree, alpha, eps, 1.0, s_nodes, True)
    ga, gat = _batch_sor(n, indptr, indices, degree, alpha, eps, 1.0, s_nodes, False)
    lo, lt = _batch_gd(n, indptr, indices, degree, alpha, eps, s_nodes, True)
    return (s_nodes, _int_opers(ls["oper"]), lst, _int_opers(gs["oper"]), gst, _int_opers(la["oper"]), lat,
            _int_opers(ga["oper"]), gat, _int_opers(lo), lt, _int_opers(go), gt)


def solve_a_graph_omega(n, indptr, indices, degree, alpha, eps, omega, graph_name, s_nodes):
    """Local SOR with omega and local APPR (omega = 1) over s_nodes (ppr_solver.py:464-508); the other entries
    of the 13-tuple stay zero, as the reference leaves them."""
    k = len(s_nodes)
    ls, lst = _batch_sor(n, indptr, indices, degree, alpha, eps, omega, s_nodes, True)
    la, lat = _batch_sor(n, indptr, indices, degree, alpha, eps, 1.0, s_nodes, True)
    z, zt = (lambda: np.zeros(k, dtype=np.int64)), (lambda: np.zeros(k))
    return (s_nodes, _int_opers(ls["oper"]), lst, z(), zt(), _int_opers(la["oper"]), lat, z(), zt(), z(), zt(), z(),
            zt())


def init_a_graph(n, indptr, indices, degree, alpha, eps, omega, graph_name, s_nodes):
    """Local SOR solutions for every seed (ppr_solver.py:696-720) -> (opers, algo_times, xs[k, n], rs[k, n])."""
    r, t = _batch_sor(n, indptr, indices, degree, alpha, eps, omega, s_nodes, True, want_x=True)
    return _int_opers(r["oper"]), t, np.asarray(r["x"], dtype=np.float64), np.asarray(r["r"], dtype=np.float64)


def updeta_graph(indptr, indices, degree, us, vs, onlyinsert=True):
    """Edge batch on the padded CSR (ppr_solver.py:723-766), on the device; indices / degree edited in place
    -> (insert_neighbor, delete_neighbor): node -> neighbours inserted / deleted, in batch order."""
    _, outcome = edit_batch(indptr, indices, degree, us, vs, onlyinsert)
    return neighbour_maps(np.asarray(us), np.asarray(vs), outcome)


def update_ppr(n, indptr, indices, degree, old_degree, p, r, alpha, queue, front, rear, q_mark, eps_vec,
               insert_neighbor, delete_neighbor, omega):
    """One feature row of the dynamic PPR update (ppr_solver.py:769-821) on the device, after updeta_graph:
    repair p, r at the nodes with insertions, then push from them (omega != 1: multicolour SOR order).
    p, r are updated in place -> (runtime, oper)."""
    g = graph_for(indptr, indices, degree, padded=True)
    eps = eps_from_vec(eps_vec, alpha * np.asarray(degree, dtype=np.float64))
    keys, old_deg, off, nbr = repair_lists(insert_neighbor, delete_neighbor, old_degree, True)
    pending = queue_entries(queue, front, rear, n + 2)
    with Timer() as t:
        oper = column_repair_push(g, L.UPPR, p, r, None, keys, old_deg, off, nbr, pending, alpha, eps, 0.0, omega)
    q_mark[:] = False
    # ppr_solver.py:778-787 counts the repair: 2 per key plus its neighbour lists
    return t.dt, int(round(oper)) + 2 * len(keys) + int(off[-1])


def update_ppr_parallel(n, indptr, indices, degree, alpha, eps, omega, P, R, us, vs, batchsize=50):
    """Dynamic PPR update (ppr_solver.py:824-849): edits the padded CSR in place, repairs and pushes.

    P, R are F x n (one row per feature) and are updated in place; returns
    (opers, runtimes, P, R).  omega != 1 relaxes in multicolour SOR order;
    omega = 1 pushes synchronously.
    """
    import torch
    assert indices.dtype == np.int32 and degree.dtype == np.int64, "indices int32 and degree int64 (as the reference)"
    g = graph_for(indptr, indices, degree, padded=True)
    dev = f"cuda:{g.ctx.device}"
    Pd = torch.from_numpy(np.ascontiguousarray(P.T)).to(dev)
    Rd = torch.from_numpy(np.ascontiguousarray(R.T)).to(dev)
    with Timer() as t:
        res = api.feature_update(g, L.UPPR, indices, degree, us, vs, False, Pd, Rd, None, eps, alpha=alpha,
                                 prec="fp64", omega=omega)
    rekey(g, indptr, indices, degree)  # the resident graph already holds the edit
    P[:] = Pd.T.cpu().numpy()
    R[:] = Rd.T.cpu().numpy()
    F = P.shape[0]
    return res["oper"].astype(np.int64), np.full(F, t.dt / max(F, 1)), P, R


def optimal_omega(alpha):
    """The reference drivers' optimal SOR weight (demo.py:31-35) -> (alpha, omega)."""
    a = alpha / (2 - alpha)
    mu = (1. - a) / (1. + a)
    omega = 1. + (mu / (1. + np.sqrt(1. - mu ** 2.))) ** 2.
    return 2 * a / (1 + a), omega
