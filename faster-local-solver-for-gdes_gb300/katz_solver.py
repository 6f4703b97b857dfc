"""Drop-in GPU replacement of the reference's ``katz_solver.py`` (Katz centrality).

    (I - alpha A) x = e_s   (katz_solver.py:177-179; returned x has x[s] -= 1 for GD)

Same names, positional arguments and return tuples as the reference; the
solves run in ``libgde.so`` on the GPU.  (The reference's module docstring
repeats the PPR system; the Katz system above is what its code solves.)
"""
from __future__ import annotations

import numpy as np

from gde import _lib as L
from gde import api
from gde.dropin import Timer, graph_for, oper_like

__all__ = ["katz_gd", "katz_gd_local_gpu", "katz_gd_standard_gpu", "katz_cheby", "solve_a_graph_gpu",
           "solve_a_graph_cheby", "katz_sor", "katz_spectral_bounds"]


def _solve1(n, indptr, indices, degree, s_node, alpha, eps, method, prec, l_max=0.0, mu_min=0.0):
    g = graph_for(indptr, indices, degree)
    assert g.n == n, "n must equal len(indptr) - 1"
    r = api.solve(g, L.KATZ, method, [s_node], [eps], prec=prec, alpha=alpha, l_max=l_max, mu_min=mu_min)
    return r["x"][0], r["r"][0], r["oper"][0]


def katz_gd(n, indptr, indices, degree, s_node, alpha, eps, local):
    """Local/global GD (katz_solver.py:167-248) -> (xt, rt, oper, algo_time)."""
    with Timer() as t:
        x, r, oper = _solve1(n, indptr, indices, degree, s_node, alpha, eps, L.LOCAL_GD if local else L.GLOBAL_GD,
                             "fp64")
    return x, r, oper_like(degree, oper), t.dt


def katz_gd_local_gpu(n, indptr, indices, degree, s_node, alpha, eps):
    """LocalGD on the GPU, FP32 (katz_solver.py:81-146)."""
    with Timer() as t:
        x, r, oper = _solve1(n, indptr, indices, degree, s_node, alpha, eps, L.LOCAL_GD, "fp32")
    return x, r, float(oper), t.dt


def katz_gd_standard_gpu(n, indptr, indices, degree, s_node, alpha, eps):
    """Global GD on the GPU, FP32 (katz_solver.py:24-78)."""
    with Timer() as t:
        x, r, oper = _solve1(n, indptr, indices, degree, s_node, alpha, eps, L.GLOBAL_GD, "fp32")
    return x, r, float(oper), t.dt


def katz_cheby(n, indptr, indices, degree, s_node, alpha, l_max, mu_min, eps, local):
    """Chebyshev with spectral bounds (katz_solver.py:340-431) -> (xt, rt, oper, algo_time)."""
    with Timer() as t:
        x, r, oper = _solve1(n, indptr, indices, degree, s_node, alpha, eps,
                             L.LOCAL_CHEBY if local else L.GLOBAL_CHEBY, "fp64", l_max, mu_min)
    return x, r, oper_like(degree, oper), t.dt


def solve_a_graph_gpu(n, indptr, indices, degree, alpha, eps, s_nodes):
    """(katz_solver.py:149-164) -> (s_nodes, local_times, global_times)."""
    test_num = len(s_nodes)
    lt = np.zeros(test_num)
    gt = np.zeros(test_num)
    for ii in range(test_num):
        gt[ii] = katz_gd_standard_gpu(n, indptr, indices, degree, int(s_nodes[ii]), alpha, eps)[3]
    for ii in range(test_num):
        lt[ii] = katz_gd_local_gpu(n, indptr, indices, degree, int(s_nodes[ii]), alpha, eps)[3]
    return s_nodes, lt, gt


def solve_a_graph_cheby(n, indptr, indices, degree, alpha, l_max, mu_min, eps, graph_name, s_nodes):
    """(katz_solver.py:669-698) -> (s_nodes, local_opers, local_times, global_opers, global_times)."""
    test_num = len(s_nodes)
    lo = np.zeros(test_num, dtype=np.int64)
    lt = np.zeros(test_num)
    go = np.zeros(test_num, dtype=np.int64)
    gt = np.zeros(test_num)
    for ii in range(test_num):
        _, _, lo[ii], lt[ii] = katz_cheby(n, indptr, indices, degree, int(s_nodes[ii]), alpha, l_max, mu_min, eps, True)
    for ii in range(test_num):
        _, _, go[ii], gt[ii] = katz_cheby(n, indptr, indices, degree, int(s_nodes[ii]), alpha, l_max, mu_min, eps,
                                          False)
    return s_nodes, lo, lt, go, gt


def katz_spectral_bounds(n, indptr, indices, degree, alpha):
    """(l_max, mu_min, lambda_max, lambda_min) for katz_cheby on the GPU.

    The reference computes lambda_max(A) and lambda_min(A) with
    scipy.sparse.linalg.eigsh in its experiment scripts (katz_exp_dmax.py:20,
    katz_exp_dmin.py:20); here a Lanczos iteration runs on the device.  The
    spectrum of Q = I - alpha A then lies in [mu_min, l_max].
    """
    g = graph_for(indptr, indices, degree)
    assert g.n == n, "n must equal len(indptr) - 1"
    b = api.katz_spectral_bounds(g, alpha)
    return b["l_max"], b["mu_min"], b["lam_max"], b["lam_min"]


def katz_sor(n, indptr, indices, degree, s_node, alpha, eps, omega, local):
    """LocalSOR / global SOR for Katz (katz_solver.py:251-337) -> (xt, rt, oper, algo_time).

    Multicolour Gauss-Seidel order on the GPU (see ``ppr_solver.ppr_sor``);
    the returned xt has xt[s_node] -= 1 like the reference's.
    """
    g = graph_for(indptr, indices, degree)
    assert g.n == n, "n must equal len(indptr) - 1"
    with Timer() as t:
        r = api.sor(g, L.KATZ, [s_node], [eps], omega=omega, local=local, alpha=alpha, prec="fp64")
    return r["x"][0], r["r"][0], oper_like(degree, r["oper"][0]), t.dt
