"""Operation counts of the GPU's parallel orders against the reference's sequential orders.

Five methods run on the GPU in an order the reference does not use, because
the reference's order is a sequential queue that no parallel schedule can
reproduce (the GPU matches the oracle's restatement of its own order
exactly; that is tested in ``test_gpu_parity.py`` and ``test_sor.py``):

* ``ppr_cheby`` / ``katz_cheby`` local (ppr_solver.py:582-661,
  katz_solver.py:340-431): a queue built during the round; the GPU's next
  frontier is every node at or above threshold after the round;
* ``ppr_sor`` / ``katz_sor`` (ppr_solver.py:331-461, katz_solver.py:251-337):
  FIFO Gauss-Seidel; the GPU sweeps a degree-ordered greedy colouring;
* ``instantGNNParallel`` (InstantGNN.py:12-71): FIFO per column; the GPU pushes
  synchronous rounds;
* ``hk_sor_queue`` local with omega != 1 (hk_solver.py:206-295): the GPU
  relaxes each node to its threshold at every level.

This file reports, on the 100k-node Chung-Lu graph (exponent 2.1, mean
degree 10, maximum 2,000), how the operation count and the error against the
FP64 truth of the GPU's order compare with the reference's order, both
computed by the oracle.  Run with ``-s`` to print the table.  The asserted bounds are wide;
the measured ratios are the point.
"""
import numpy as np
import pytest

from oracle import oracle as O
from gde import graphs

ALPHA = 0.1


@pytest.fixture(scope="module")
def c1():
    g = graphs.chung_lu_100k()
    return g, g.degree.astype(np.float64)


def _row(name, o_ref, o_gpu, e_ref=None, e_gpu=None):
    ratio = o_gpu / o_ref
    err = "" if e_ref is None else f"  l1 vs truth: reference {e_ref:.3e}, GPU order {e_gpu:.3e}"
    print(f"{name:34s} opers reference {o_ref:14.0f}  GPU order {o_gpu:14.0f}  ratio {ratio:6.3f}{err}")
    return ratio


def test_ppr_cheby_and_sor_orders(c1):
    g, deg = c1
    seeds = graphs.uniform_seeds(g, 4, seed=21)
    order = np.argsort(-g.degree, kind="stable")
    colors = O.greedy_colors(g.indptr, g.indices, order)
    eps = 1e-6
    print()
    for s in seeds:
        s = int(s)
        truth = O.global_solve_ppr(g.indptr, g.indices, deg, s, ALPHA)
        xq, _, oq = O.cheby(g.n, g.indptr, g.indices, deg, s, ALPHA, eps, True)
        xs, _, os_ = O.cheby(g.n, g.indptr, g.indices, deg, s, ALPHA, eps, True, sync=True)
        r = _row(f"ppr_cheby local, seed {s}", oq, os_, np.abs(xq - truth).sum(), np.abs(xs - truth).sum())
        assert 0.25 < r < 2.0
        assert np.abs(xs - truth).sum() < 2 * np.abs(xq - truth).sum() + 1e-9
        xf, _, of = O.sor(g.n, g.indptr, g.indices, deg, s, ALPHA, eps, 1.3, True)
        xc, _, oc, _ = O.sor_color(g.n, g.indptr, g.indices, deg, s, ALPHA, eps, 1.3, True, colors)
        r = _row(f"ppr_sor omega 1.3, seed {s}", of, oc, np.abs(xf - truth).sum(), np.abs(xc - truth).sum())
        assert 0.5 < r < 2.0
        assert np.abs(xc - truth).sum() < 2 * np.abs(xf - truth).sum() + 1e-9


def test_katz_cheby_and_sor_orders(c1):
    g, deg = c1
    import scipy.sparse as sp
    from scipy.sparse.linalg import eigsh
    A = sp.csr_matrix((np.ones(g.nnz), g.indices, g.indptr), shape=(g.n, g.n))
    lam_max = float(eigsh(A, k=1, which="LA", return_eigenvectors=False, tol=1e-8)[0])
    lam_min = float(eigsh(A, k=1, which="SA", return_eigenvectors=False, tol=1e-8)[0])
    alpha = 0.5 / float(g.degree.max())
    l_max, mu_min = 1.0 - alpha * lam_min, 1.0 - alpha * lam_max
    order = np.argsort(-g.degree, kind="stable")
    colors = O.greedy_colors(g.indptr, g.indices, order)
    eps = 1e-7
    print()
    for s in graphs.uniform_seeds(g, 3, seed=22):
        s = int(s)
        xq, _, oq = O.cheby(g.n, g.indptr, g.indices, deg, s, alpha, eps, True, katz=True, l_max=l_max,
                            mu_min=mu_min)
        xs, _, os_ = O.cheby(g.n, g.indptr, g.indices, deg, s, alpha, eps, True, katz=True, l_max=l_max,
                             mu_min=mu_min, sync=True)
        r = _row(f"katz_cheby local, seed {s}", oq, os_)
        print(f"{'':34s} l1 between the two orders {np.abs(xq - xs).sum():.3e} (sum x {xq.sum():.4f})")
        assert 0.5 < r < 2.0
        xf, _, of = O.sor(g.n, g.indptr, g.indices, deg, s, alpha, eps, 1.1, True, katz=True)
        xc, _, oc, _ = O.sor_color(g.n, g.indptr, g.indices, deg, s, alpha, eps, 1.1, True, colors, katz=True)
        r = _row(f"katz_sor omega 1.1, seed {s}", of, oc)
        print(f"{'':34s} l1 between the two orders {np.abs(xf - xc).sum():.3e}")
        assert 0.5 < r < 2.0


def test_instantgnn_static_order(c1):
    g, deg = c1
    rng = np.random.default_rng(23)
    F = 4
    X = rng.standard_normal((g.n, F))
    beta, eps = 0.5, 1e-6
    P0, R0 = np.zeros((g.n, F)), X.copy()
    Pf, Rf = P0.copy(), R0.copy()
    ofifo = O.ign_static(g.n, g.indptr, g.indices, g.degree, ALPHA, eps, Pf, Rf, beta)
    Ps, Rs = P0.copy(), R0.copy()
    osync = O.ign_sync(g.n, g.indptr, g.indices, g.degree, ALPHA, eps, beta, Ps, Rs)
    eps_vec = np.power(deg, 1 - beta) * eps
    assert (np.abs(Rs) < eps_vec[:, None]).all()
    assert (np.abs(Rf) < eps_vec[:, None]).all()
    # the reference keeps p in float32 (InstantGNN.py:55), so the two orders
    # differ by that rounding as well as by the order
    d = np.abs(Pf - Ps).sum(axis=0) / np.abs(Pf).sum(axis=0)
    print()
    for f in range(F):
        r = _row(f"instantGNN column {f}", ofifo[f], osync[f])
        print(f"{'':34s} relative l1 between the two orders {d[f]:.3e}")
        assert 0.5 < r < 4.0
        assert d[f] < 1e-3
    assert (d < 1e-3).all()


def test_hk_relaxed_local_order(c1):
    g, deg = c1
    tau, eps, omega = 5.0, 1e-6, 1.3
    print()
    for s in graphs.uniform_seeds(g, 2, seed=24):
        s = int(s)
        _, xq, _, oq = O.hk_sor_queue(g.n, g.indptr, g.indices, deg, s, tau, eps, omega, True)
        _, xs, _, os_ = O.hk_sor_queue(g.n, g.indptr, g.indices, deg, s, tau, eps, omega, True, sync=True)
        r = _row(f"hk_sor_queue local omega 1.3, seed {s}", oq, os_)
        print(f"{'':34s} sum x: reference {xq.sum():.4f}, GPU order {xs.sum():.4f} (the heat kernel sums to 1)")
        assert 1.0 <= r < 8.0
        assert abs(xs.sum() - 1.0) < abs(xq.sum() - 1.0) + 1e-3
