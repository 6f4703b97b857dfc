"""Drop-in GPU replacement of the reference's ``katz_solver.py`` (Katz centrality).

    (I - alpha A) x = e_s   (katz_solver.py:177-179; returned x has x[s] -= 1 for GD)

Same names, positional arguments and return tuples as the reference; the
solves run in ``libgde.so`` on the GPU.  The ``solve_a_graph_*`` drivers
solve all their seeds in one batched call per method; each seed's
``algo_time`` is that call's wall time divided by the number of seeds.  (The reference's module docstring
repeats the PPR system; the Katz system above is what its code solves.)
"""
from __future__ import annotations

import numpy as np

from gde import _lib as L
from gde import api
from gde.dropin import Timer, graph_for, oper_like

__all__ = ["katz_gd", "katz_gd_local_gpu", "katz_gd_standard_gpu", "katz_cheby", "solve_a_graph_gpu",
           "solve_a_graph_cheby", "katz_sor", "katz_spectral_bounds", "solve_a_graph_all", "solve_a_graph_omega",
           "solve_a_graph_ratio", "solve_a_graph_pk"]


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


def _seeds(s_nodes) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(s_nodes).ravel(), dtype=np.int32)


def _per_seed(dt: float, k: int) -> np.ndarray:
    return np.full(k, dt / max(k, 1))


def _int_opers(oper) -> np.ndarray:
    return np.rint(np.asarray(oper, dtype=np.float64)).astype(np.int64)


def _graph(n, indptr, indices, degree):
    g = graph_for(indptr, indices, degree)
    assert g.n == n, "n must equal len(indptr) - 1"
    return g


def _batch(n, indptr, indices, degree, alpha, eps, s_nodes, method, prec="fp64", l_max=0.0, mu_min=0.0):
    """(opers, per-seed times) of one Katz method over s_nodes in one batched solve."""
    g = _graph(n, indptr, indices, degree)
    seeds = _seeds(s_nodes)
    with Timer() as t:
        r = api.solve(g, L.KATZ, method, seeds, eps, prec=prec, alpha=alpha, l_max=l_max, mu_min=mu_min,
                      want_x=False, want_r=False)
    return r["oper"], _per_seed(t.dt, len(seeds))


def _batch_sor(n, indptr, indices, degree, alpha, eps, omega, s_nodes, local, device_x=False):
    g = _graph(n, indptr, indices, degree)
    seeds = _seeds(s_nodes)
    with Timer() as t:
        r = api.sor(g, L.KATZ, seeds, eps, omega=omega, local=local, alpha=alpha, prec="fp64", want_x=device_x,
                    want_r=False, device_out=device_x)
    return r, _per_seed(t.dt, len(seeds))


def solve_a_graph_gpu(n, indptr, indices, degree, alpha, eps, s_nodes):
    """GPU global then local GD over s_nodes, FP32 (katz_solver.py:149-164) -> (s_nodes, local_times, global_times)."""
    _, gt = _batch(n, indptr, indices, degree, alpha, eps, s_nodes, L.GLOBAL_GD, "fp32")
    _, lt = _batch(n, indptr, indices, degree, alpha, eps, s_nodes, L.LOCAL_GD, "fp32")
    return s_nodes, lt, gt


def solve_a_graph_cheby(n, indptr, indices, degree, alpha, l_max, mu_min, eps, graph_name, s_nodes):
    """(katz_solver.py:669-698) -> (s_nodes, local_opers, local_times, global_opers, global_times)."""
    lo, lt = _batch(n, indptr, indices, degree, alpha, eps, s_nodes, L.LOCAL_CHEBY, l_max=l_max, mu_min=mu_min)
    go, gt = _batch(n, indptr, indices, degree, alpha, eps, s_nodes, L.GLOBAL_CHEBY, l_max=l_max, mu_min=mu_min)
    return s_nodes, _int_opers(lo), lt, _int_opers(go), gt


def _all_methods(n, indptr, indices, degree, alpha, eps, omega, s_nodes):
    ls, lst = _batch_sor(n, indptr, indices, degree, alpha, eps, omega, s_nodes, True)
    gs, gst = _batch_sor(n, indptr, indices, degree, alpha, eps, omega, s_nodes, False)
    la, lat = _batch_sor(n, indptr, indices, degree, alpha, eps, 1.0, s_nodes, True)
    ga, gat = _batch_sor(n, indptr, indices, degree, alpha, eps, 1.0, s_nodes, False)
    lo, lt = _batch(n, indptr, indices, degree, alpha, eps, s_nodes, L.LOCAL_GD)
    go, gt = _batch(n, indptr, indices, degree, alpha, eps, s_nodes, L.GLOBAL_GD)
    return (ls["oper"], lst, gs["oper"], gst, la["oper"], lat, ga["oper"], gat, lo, lt, go, gt)


def solve_a_graph_all(n, indptr, indices, degree, alpha, eps, omega, graph_name, s_nodes):
    """Every Katz method over s_nodes (katz_solver.py:605-666): local / global SOR with omega, local / global
    AKatz (omega = 1), local / global GD -> (s_nodes, local_sor_opers, local_sor_algo_times, global_sor_opers,
    global_sor_algo_times, local_akatz_opers, local_akatz_algo_times, global_akatz_opers,
    global_akatz_algo_times, local_gd_opers, local_gd_algo_times, global_gd_opers, global_gd_algo_times)."""
    r = _all_methods(n, indptr, indices, degree, alpha, eps, omega, s_nodes)
    return (s_nodes, *[_int_opers(v) if i % 2 == 0 else v for i, v in enumerate(r)])


def solve_a_graph_omega(n, indptr, indices, degree, alpha, eps, omega, graph_name, s_nodes):
    """Local SOR with omega over s_nodes (katz_solver.py:561-602); the other entries stay zero, as the
    reference leaves them."""
    k = len(s_nodes)
    ls, lst = _batch_sor(n, indptr, indices, degree, alpha, eps, omega, s_nodes, True)
    z, zt = (lambda: np.zeros(k, dtype=np.int64)), (lambda: np.zeros(k))
    return (s_nodes, _int_opers(ls["oper"]), lst, z(), zt(), z(), zt(), z(), zt(), z(), zt(), z(), zt())


def solve_a_graph_ratio(n, indptr, indices, degree, alpha, eps, omega, graph_name, s_nodes):
    """Global-to-local work and time ratios and per-method means (katz_solver.py:434-533) -> (n + m,
    sor oper ratio, sor time ratio, akatz oper ratio, akatz time ratio, gd oper ratio, gd time ratio, then the
    mean opers and times of local SOR, global SOR, local AKatz, global AKatz, local GD and global GD)."""
    ls, lst, gs, gst, la, lat, ga, gat, lo, lt, go, gt = _all_methods(n, indptr, indices, degree, alpha, eps, omega,
                                                                      s_nodes)
    m = np.asarray(degree).sum()
    return (n + m, (gs / ls).mean(), (gst / lst).mean(), (ga / la).mean(), (gat / lat).mean(), (go / lo).mean(),
            (gt / lt).mean(), ls.mean(), lst.mean(), gs.mean(), gst.mean(), la.mean(), lat.mean(), ga.mean(),
            gat.mean(), lo.mean(), lt.mean(), go.mean(), gt.mean())


def solve_a_graph_pk(n, indptr, indices, degree, alpha, eps, omega, graph_name, s_nodes):
    """Local SOR over s_nodes and each solution's participation ratio
    pk = (sum (n x)^2)^2 / sum (n x)^4 (katz_solver.py:536-558) -> (opers, algo_times, pk)."""
    r, t = _batch_sor(n, indptr, indices, degree, alpha, eps, omega, s_nodes, True, device_x=True)
    xn = r["x"].double() * n
    sq = (xn * xn)
    pk = ((sq.sum(1) ** 2) / (sq * sq).sum(1)).cpu().numpy()
    return np.asarray(r["oper"], dtype=np.float64), t, pk


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
