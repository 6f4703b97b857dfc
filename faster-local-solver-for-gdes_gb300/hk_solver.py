"""Drop-in GPU replacement of the reference's ``hk_solver.py`` (heat kernel).

    h = e^{-tau} sum_k tau^k/k! (A D^{-1})^k e_s, truncated at N = estimate_n(tau, eps/2)

``hk_sor_queue`` runs the level-synchronous push on the GPU: level j's
active nodes move r_j into x and push tau/(j+1) r_j/d into level j+1; the
last level pushes r/d straight into x (hk_solver.py:235-295).  With a
relaxation omega != 1 a node moves omega r and keeps r - omega r at its
level, and relaxes again while that stays at or above its threshold
(hk_solver.py:248-264); the global form sweeps all nodes together as the
reference does (:266-280).
``hk_taylor_approx`` is the global Taylor series (hk_solver.py:51-80).
"""
from __future__ import annotations

import numpy as np

from gde import _lib as L
from gde import api
from gde.dropin import Timer, graph_for

__all__ = ["estimate_coefficient", "estimate_n", "hk_taylor_approx", "hk_sor_queue", "solve_a_graph_all",
           "solve_a_graph_pk"]


def estimate_coefficient(t, k):
    """t^{k+1}/(k+1)!, k >= 0, t >= 1 (hk_solver.py:15-25)."""
    assert k >= 0
    assert t >= 1.
    t0 = t
    for i in range(int(k)):
        t0 = t0 * (t / (i + 2))
    return t0


def estimate_n(t, eps):
    """Taylor length N with ||D^-1 h - D^-1 y|| <= eps (hk_solver.py:28-48), computed in libgde."""
    assert t >= 1.
    assert eps > 0.
    return api.hk_estimate_n(t, eps)


def hk_taylor_approx(n, indptr, indices, degree, s_node, tau, eps):
    """Global Taylor approximation (hk_solver.py:51-80) -> (est_n, xt, algo_time)."""
    assert tau >= 1.
    assert eps >= 0.
    g = graph_for(indptr, indices, degree)
    with Timer() as t:
        r = api.solve(g, L.HK, L.HK_TAYLOR, [s_node], [eps], prec="fp64", tau=tau, want_r=False)
    return estimate_n(tau, eps), r["x"][0], t.dt


def hk_sor_queue(n, indptr, indices, degree, s_node, tau, eps, omega, local):
    """Level push (hk_solver.py:206-295) -> (est_n, xt, rt[2, n], oper, beta_t, run_time, algo_time).

    omega = 1 and the global form (local=False) give the reference's result.
    The local form with omega != 1 relaxes every node at or above threshold
    until its kept residual drops below it.  The reference's queue instead
    re-enqueues a node only if it is not yet queued for the next level
    (hk_solver.py:262), a test that depends on the queue order and that
    leaves most of (1 - omega) r unpushed.  beta_t is not tracked by the GPU
    path and is returned empty.
    """
    g = graph_for(indptr, indices, degree)
    with Timer() as t:
        r = api.solve(g, L.HK, L.HK_LOCAL if local else L.HK_GLOBAL, [s_node], [eps], prec="fp64", tau=tau,
                      omega=float(omega))
    est_n = estimate_n(tau, .5 * eps)
    return est_n, r["x"][0], r["r"][0], float(r["oper"][0]), [], t.dt, t.dt


def _batch(n, indptr, indices, degree, s_nodes, tau, eps, omega, local, device_x=False):
    g = graph_for(indptr, indices, degree)
    assert g.n == n, "n must equal len(indptr) - 1"
    seeds = np.ascontiguousarray(np.asarray(s_nodes).ravel(), dtype=np.int32)
    with Timer() as t:
        r = api.solve(g, L.HK, L.HK_LOCAL if local else L.HK_GLOBAL, seeds, eps, prec="fp64", tau=tau,
                      omega=float(omega), want_x=device_x, want_r=False, device_out=device_x)
    return r, np.full(len(seeds), t.dt / max(len(seeds), 1))


def solve_a_graph_all(n, indptr, indices, degree, tau, eps, omega, graph_name, s_nodes):
    """(hk_solver.py:303-366): local and global SOR with ``omega``, then the omega = 1 ("ahk") pair, each
    over all seeds in one batched call.  The Taylor and relax entries stay zero, as the reference leaves them.
    """
    test_num = len(s_nodes)
    z = lambda: np.zeros(test_num, dtype=np.int64)  # noqa: E731
    zt = lambda: np.zeros(test_num)  # noqa: E731
    out = []
    for om, local in ((omega, True), (omega, False), (1.0, True), (1.0, False)):
        r, t = _batch(n, indptr, indices, degree, s_nodes, tau, eps, om, local)
        out += [np.rint(r["oper"]).astype(np.int64), t]
    return (s_nodes, *out, z(), zt(), z(), zt())


def solve_a_graph_pk(n, indptr, indices, degree, tau, eps, omega, graph_name, s_nodes):
    """Global level push (omega = 1) over s_nodes with each solution's participation ratio
    pk = (sum (n x)^2)^2 / sum (n x)^4 (hk_solver.py:369-393) -> (opers, algo_times, pk, est_ns)."""
    r, t = _batch(n, indptr, indices, degree, s_nodes, tau, eps, 1.0, False, device_x=True)
    xn = r["x"].double() * n
    sq = xn * xn
    pk = ((sq.sum(1) ** 2) / (sq * sq).sum(1)).cpu().numpy()
    est = np.full(len(s_nodes), float(estimate_n(tau, .5 * eps)))
    return np.asarray(r["oper"], dtype=np.float64), t, pk, est
