"""Drop-in GPU replacement of the reference's ``ppr_solver.py`` (personalized PageRank).

    Q x = b,  Q = I - (1-alpha) A D^{-1},  b = alpha e_s   (ppr_solver.py:18-23)

Same function names, positional arguments and return tuples as the
reference; every solve runs in ``libgde.so`` on the GPU (synchronous local
push, ``csrc/push_engine.cu``).  FP64 functions return float64 arrays;
the ``*_gpu`` functions compute in FP32 residuals with a Kahan-compensated
FP32 solution, like the reference's CuPy path returns float32.
"""
from __future__ import annotations

import numpy as np

from gde import _lib as L
from gde import api
from gde.dropin import Timer, graph_for, oper_like

__all__ = ["ppr_gd", "ppr_gd_local_gpu", "ppr_gd_standard_gpu", "ppr_cheby", "ppr_sor", "ppr_gd_torch",
           "solve_a_graph_gpu", "solve_a_graph_cheby", "solve_a_graph_torch", "update_ppr_parallel", "optimal_omega"]


def _solve1(n, indptr, indices, degree, s_node, alpha, eps, method, prec):
    g = graph_for(indptr, indices, degree)
    assert g.n == n, "n must equal len(indptr) - 1"
    r = api.solve(g, L.PPR, method, [s_node], [eps], prec=prec, alpha=alpha)
    return r["x"][0], r["r"][0], r["oper"][0]


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
    """Mean time of the global reference solve over s_nodes (ppr_solver.py:191-205)."""
    times = []
    for s in s_nodes:
        with Timer() as t:
            _solve1(n, indptr, indices, degree, int(s), alpha, eps, L.GLOBAL_GD, "fp64")
        times.append(t.dt)
    return float(np.mean(times))


def solve_a_graph_gpu(n, indptr, indices, degree, alpha, eps, s_nodes):
    """Per-seed GPU global then local GD times (ppr_solver.py:149-164) -> (s_nodes, local_times, global_times)."""
    test_num = len(s_nodes)
    local_t = np.zeros(test_num)
    global_t = np.zeros(test_num)
    for ii in range(test_num):
        global_t[ii] = ppr_gd_standard_gpu(n, indptr, indices, degree, int(s_nodes[ii]), alpha, eps)[3]
    for ii in range(test_num):
        local_t[ii] = ppr_gd_local_gpu(n, indptr, indices, degree, int(s_nodes[ii]), alpha, eps)[3]
    return s_nodes, local_t, global_t


def solve_a_graph_cheby(n, indptr, indices, degree, alpha, eps, omega, graph_name, s_nodes):
    """Local and global Chebyshev over s_nodes (ppr_solver.py:664-693)."""
    test_num = len(s_nodes)
    lo = np.zeros(test_num, dtype=np.int64)
    lt = np.zeros(test_num)
    go = np.zeros(test_num, dtype=np.int64)
    gt = np.zeros(test_num)
    for ii in range(test_num):
        _, _, lo[ii], lt[ii] = ppr_cheby(n, indptr, indices, degree, int(s_nodes[ii]), alpha, eps, True)
    for ii in range(test_num):
        _, _, go[ii], gt[ii] = ppr_cheby(n, indptr, indices, degree, int(s_nodes[ii]), alpha, eps, False)
    return s_nodes, lo, lt, go, gt


def update_ppr_parallel(n, indptr, indices, degree, alpha, eps, omega, P, R, us, vs, batchsize=50):
    """Dynamic PPR update (ppr_solver.py:824-849): edits the padded CSR in place, repairs and pushes.

    P, R are F x n (one row per feature) and are updated in place; returns
    (opers, runtimes, P, R).  omega != 1 relaxes in multicolour SOR order;
    omega = 1 pushes synchronously.
    """
    import torch
    g = graph_for(indptr, indices, degree, padded=True)
    dev = f"cuda:{g.ctx.device}"
    Pd = torch.from_numpy(np.ascontiguousarray(P.T)).to(dev)
    Rd = torch.from_numpy(np.ascontiguousarray(R.T)).to(dev)
    with Timer() as t:
        res = api.feature_update(g, L.UPPR, indices, degree, us, vs, False, Pd, Rd, None, eps, alpha=alpha,
                                 prec="fp64", omega=omega)
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
