"""The four drop-in modules, called the way the reference's callers call them.

Every exported name of ``ppr_solver``, ``katz_solver``, ``hk_solver`` and
``InstantGNN`` is called with the reference's positional arguments on small
graphs and compared with the oracle (FP64: the reference's operation counts
exactly, solutions to 1e-12; reordered methods: the oracle's restatement of
the GPU's order).  The last tests run the call sequences of the reference's
drivers (``demo.py:39-56``, ``test_epsilon.py:40-50``) unmodified against a
small synthetic graph saved as ``<name>_csr-mat.npz``.
"""
import numpy as np
import pytest

from gde import _lib as L
from gde import api, graphs
from oracle import oracle as O

from test_device_edit import _mixed_batch, _padded

pytestmark = pytest.mark.gpu

ALPHA = 0.15


@pytest.fixture(scope="module")
def mods():
    import hk_solver
    import InstantGNN
    import katz_solver
    import ppr_solver
    return ppr_solver, katz_solver, hk_solver, InstantGNN


@pytest.fixture(scope="module")
def cl():
    g = graphs.chung_lu(2500, 2.1, 8.0, 250.0, seed=13)
    return g, g.indptr.astype(np.int64), g.indices.astype(np.int32), g.degree.astype(np.int64)


def colors_of(indptr, indices, degree):
    return api.graph_colors(api.Graph(indptr, indices, degree=np.asarray(degree, np.float64)))


def test_every_exported_name_is_callable(mods):
    expect = {
        "ppr_solver": {"ppr_gd", "ppr_gd_local_gpu", "ppr_gd_standard_gpu", "ppr_cheby", "ppr_sor", "ppr_gd_torch",
                       "solve_a_graph_gpu", "solve_a_graph_cheby", "solve_a_graph_torch", "solve_a_graph_all",
                       "solve_a_graph_omega", "init_a_graph", "updeta_graph", "update_ppr", "update_ppr_parallel"},
        "katz_solver": {"katz_gd", "katz_gd_local_gpu", "katz_gd_standard_gpu", "katz_cheby", "katz_sor",
                        "solve_a_graph_gpu", "solve_a_graph_cheby", "solve_a_graph_all", "solve_a_graph_omega",
                        "solve_a_graph_ratio", "solve_a_graph_pk"},
        "hk_solver": {"estimate_coefficient", "estimate_n", "hk_taylor_approx", "hk_sor_queue", "solve_a_graph_all",
                      "solve_a_graph_pk"},
        "InstantGNN": {"instantGNNPush", "instantGNNParallel", "instantGNNSorPush", "instantGNNSorParallel",
                       "updetaGraph", "instantGNNUpdateBatch", "instantGNNUpdateBatchParallel"},
    }
    for m in mods:
        assert expect[m.__name__] <= set(m.__all__), (m.__name__, expect[m.__name__] - set(m.__all__))
        for name in m.__all__:
            assert callable(getattr(m, name))


def test_ppr_single_query_functions(mods, cl):
    ppr, _, _, _ = mods
    g, ip, ix, dg = cl
    n, s, eps = g.n, int(graphs.uniform_seeds(g, 1, seed=1)[0]), 1e-6
    for local in (True, False):
        x, r, oper, t = ppr.ppr_gd(n, ip, ix, dg, s, ALPHA, eps, local, None)
        xo, ro, oo = O.ppr_gd(n, ip, ix, dg, s, ALPHA, eps, local)
        assert isinstance(oper, int) and oper == oo and t > 0
        assert np.abs(x - xo).sum() < 1e-12 and np.abs(r - ro).sum() < 1e-12
        x, r, oper, t = ppr.ppr_cheby(n, ip, ix, dg, s, ALPHA, eps, local)
        xc, _, oc = O.cheby(n, ip, ix, dg, s, ALPHA, eps, local, sync=True)
        assert oper == oc and np.abs(x - xc).sum() < 1e-10
    for fn, local in ((ppr.ppr_gd_local_gpu, True), (ppr.ppr_gd_standard_gpu, False)):
        xo, _, oo = O.ppr_gd(n, ip, ix, dg, s, ALPHA, eps, local)
        x, r, oper, t = fn(n, ip, ix, dg, s, ALPHA, eps)
        assert x.dtype == np.float32 and np.abs(x.astype(np.float64) - xo).sum() < 1e-4
    col = colors_of(ip, ix, dg)
    omega = ppr.optimal_omega(ALPHA)[1]
    for local in (True, False):
        x, r, oper, t = ppr.ppr_sor(n, ip, ix, dg, s, ALPHA, eps, omega, local, None)
        xs, _, os_, _ = O.sor_color(n, ip, ix, dg, s, ALPHA, eps, omega, local, col)
        assert oper == int(os_) and np.abs(x - xs).sum() < 1e-10


def test_ppr_solve_a_graph_drivers(mods, cl):
    ppr, _, _, _ = mods
    g, ip, ix, dg = cl
    n, eps = g.n, 1e-6
    s_nodes = graphs.uniform_seeds(g, 6, seed=2)
    omega = ppr.optimal_omega(ALPHA)[1]
    col = colors_of(ip, ix, dg)
    res = ppr.solve_a_graph_all(n, ip, ix, dg, ALPHA, eps, omega, "synthetic", s_nodes)
    assert len(res) == 13 and res[0] is s_nodes
    for i in range(1, 13, 2):
        assert res[i].dtype == np.int64 and res[i].shape == (6,) and (res[i + 1] > 0).all()
    for j, s in enumerate(s_nodes):
        s = int(s)
        assert res[9][j] == O.ppr_gd(n, ip, ix, dg, s, ALPHA, eps, True)[2]
        assert res[11][j] == O.ppr_gd(n, ip, ix, dg, s, ALPHA, eps, False)[2]
        for k, (om, local) in enumerate(((omega, True), (omega, False), (1.0, True), (1.0, False))):
            assert res[1 + 2 * k][j] == int(O.sor_color(n, ip, ix, dg, s, ALPHA, eps, om, local, col)[2]), (k, j)
    om = ppr.solve_a_graph_omega(n, ip, ix, dg, ALPHA, eps, omega, "synthetic", s_nodes)
    np.testing.assert_array_equal(om[1], res[1])
    np.testing.assert_array_equal(om[5], res[5])
    assert not om[3].any() and not om[9].any()
    opers, times, xs, rs = ppr.init_a_graph(n, ip, ix, dg, ALPHA, eps, omega, "synthetic", s_nodes)
    np.testing.assert_array_equal(opers, res[1])
    assert xs.shape == (6, n) and rs.shape == (6, n)
    xo, ro, _, _ = O.sor_color(n, ip, ix, dg, int(s_nodes[0]), ALPHA, eps, omega, True, col)
    assert np.abs(xs[0] - xo).sum() < 1e-10 and np.abs(rs[0] - ro).sum() < 1e-10
    ch = ppr.solve_a_graph_cheby(n, ip, ix, dg, ALPHA, eps, omega, "synthetic", s_nodes)
    for j, s in enumerate(s_nodes):
        assert ch[1][j] == O.cheby(n, ip, ix, dg, int(s), ALPHA, eps, True, sync=True)[2]
        assert ch[3][j] == O.cheby(n, ip, ix, dg, int(s), ALPHA, eps, False, sync=True)[2]
    sn, lt, gt = ppr.solve_a_graph_gpu(n, ip, ix, dg, ALPHA, eps, s_nodes)
    assert sn is s_nodes and (lt > 0).all() and (gt > 0).all()
    assert ppr.solve_a_graph_torch(n, ip, ix, dg, ALPHA, eps, s_nodes, "cuda:0") > 0


def _maps(keys, off, nbr):
    return {int(k): [int(v) for v in nbr[off[i]:off[i + 1]]] for i, k in enumerate(keys)}


def test_updeta_graph_and_update_ppr(mods):
    ppr, _, _, _ = mods
    g = graphs.chung_lu(2000, 2.2, 6.0, 100.0, seed=17)
    us, vs = _mixed_batch(g, 150, 150, 40, seed=3)
    ip, ix, dg = _padded(g, 32)
    n = g.n
    # oracle: the sequential edit and the synchronous update push, row per feature
    ixo, dgo = ix.copy(), dg.copy()
    F = 3
    rng = np.random.default_rng(5)
    P0 = np.zeros((F, n))
    R0 = np.zeros((F, n))
    for f, s in enumerate(graphs.uniform_seeds(g, F, seed=6)):
        R0[f, s] = ALPHA
    O.update_ppr(n, ip, ixo, dgo, ALPHA, 1e-5, 1.0, P0, R0, np.zeros(0, np.int32), np.zeros(0, np.int32), sync=True)
    Po, Ro = P0.copy(), R0.copy()
    ixe, dge = ixo.copy(), dgo.copy()
    maps = O.update_graph(n, ip, ixe, dge, us.astype(np.int64), vs.astype(np.int64), False)
    ixo2, dgo2 = ixo.copy(), dgo.copy()
    oo = O.update_ppr(n, ip, ixo2, dgo2, ALPHA, 1e-5, 1.0, Po, Ro, us, vs, sync=True)
    # drop-in: updeta_graph edits the arrays in place and returns the neighbour maps
    ixd, dgd = ixo.copy(), dgo.copy()
    old_degree = dgd.copy()
    ins, dele = ppr.updeta_graph(ip, ixd, dgd, us, vs, onlyinsert=False)
    np.testing.assert_array_equal(ixd, ixe)
    np.testing.assert_array_equal(dgd, dge)
    assert ins == _maps(*maps[:3]) and dele == _maps(*maps[3:])
    assert list(ins) == [int(k) for k in maps[0]]  # same key order (first insertion)
    eps_vec = ALPHA * 1e-5 * dgd
    for f in range(F):
        p, r = P0[f].copy(), R0[f].copy()
        q = np.zeros(n + 2, np.int64)
        rt, oper = ppr.update_ppr(n, ip, ixd, dgd, old_degree, p, r, ALPHA, q, 0, 0, np.zeros(n), eps_vec, ins, dele,
                                  1.0)
        assert oper == oo[f], (f, oper, oo[f])
        np.testing.assert_allclose(p, Po[f], rtol=1e-9, atol=1e-13)
        np.testing.assert_allclose(r, Ro[f], rtol=1e-9, atol=1e-13)
    # update_ppr_parallel on fresh copies gives the same rows
    ixp, dgp = ixo.copy(), dgo.copy()
    P, R = P0.copy(), R0.copy()
    opers, runtimes, P, R = ppr.update_ppr_parallel(n, ip, ixp, dgp, ALPHA, 1e-5, 1.0, P, R, us, vs)
    np.testing.assert_array_equal(opers, oo)
    np.testing.assert_allclose(P, Po, rtol=1e-9, atol=1e-13)
    # the edited arrays stay bound to the edited device graph: a second batch
    us2, vs2 = _mixed_batch(g, 50, 50, 10, seed=4)
    oo2 = O.update_ppr(n, ip, ixo2, dgo2, ALPHA, 1e-5, 1.0, Po, Ro, us2, vs2, sync=True)
    opers2, _, P, R = ppr.update_ppr_parallel(n, ip, ixp, dgp, ALPHA, 1e-5, 1.0, P, R, us2, vs2)
    np.testing.assert_array_equal(ixp, ixo2)
    np.testing.assert_array_equal(opers2, oo2)
    np.testing.assert_allclose(P, Po, rtol=1e-9, atol=1e-13)


def test_katz_functions(mods, cl):
    _, katz, _, _ = mods
    g, ip, ix, dg = cl
    n, eps = g.n, 1e-6
    alpha = 1.0 / (float(dg.max()) + 1.0)
    s_nodes = graphs.uniform_seeds(g, 4, seed=8)
    s = int(s_nodes[0])
    for local in (True, False):
        x, r, oper, _ = katz.katz_gd(n, ip, ix, dg, s, alpha, eps, local)
        xo, ro, oo = O.katz_gd(n, ip, ix, dg, s, alpha, eps, local)
        assert oper == oo and np.abs(x - xo).sum() < 1e-11
    for fn, local in ((katz.katz_gd_local_gpu, True), (katz.katz_gd_standard_gpu, False)):
        x, _, _, _ = fn(n, ip, ix, dg, s, alpha, eps)
        assert np.abs(x.astype(np.float64) - O.katz_gd(n, ip, ix, dg, s, alpha, eps, local)[0]).sum() < 1e-4
    l_max, mu_min, lam_max, lam_min = katz.katz_spectral_bounds(n, ip, ix, dg, alpha)
    assert lam_min < 0 < lam_max <= dg.max()
    x, _, oper, _ = katz.katz_cheby(n, ip, ix, dg, s, alpha, l_max, mu_min, eps, True)
    xo, _, oo = O.cheby(n, ip, ix, dg, s, alpha, eps, True, katz=True, l_max=l_max, mu_min=mu_min, sync=True)
    assert oper == oo and np.abs(x - xo).sum() < 1e-10
    col = colors_of(ip, ix, dg)
    omega = 1.1
    res = katz.solve_a_graph_all(n, ip, ix, dg, alpha, eps, omega, "synthetic", s_nodes)
    assert len(res) == 13
    for j, sj in enumerate(s_nodes):
        sj = int(sj)
        assert res[9][j] == O.katz_gd(n, ip, ix, dg, sj, alpha, eps, True)[2]
        assert res[11][j] == O.katz_gd(n, ip, ix, dg, sj, alpha, eps, False)[2]
        for k, (om, local) in enumerate(((omega, True), (omega, False), (1.0, True), (1.0, False))):
            assert res[1 + 2 * k][j] == int(O.sor_color(n, ip, ix, dg, sj, alpha, eps, om, local, col, katz=True)[2])
    om = katz.solve_a_graph_omega(n, ip, ix, dg, alpha, eps, omega, "synthetic", s_nodes)
    np.testing.assert_array_equal(om[1], res[1])
    ratio = katz.solve_a_graph_ratio(n, ip, ix, dg, alpha, eps, omega, "synthetic", s_nodes)
    assert len(ratio) == 19 and ratio[0] == n + dg.sum()
    assert ratio[5] == pytest.approx((res[11] / res[9]).mean())
    opers, times, pk = katz.solve_a_graph_pk(n, ip, ix, dg, alpha, eps, omega, "synthetic", s_nodes)
    xo, _, _, _ = O.sor_color(n, ip, ix, dg, int(s_nodes[0]), alpha, eps, omega, True, col, katz=True)
    x1 = xo * n
    assert pk[0] == pytest.approx(((x1 ** 2).sum() ** 2) / (x1 ** 4).sum(), rel=1e-9)
    ch = katz.solve_a_graph_cheby(n, ip, ix, dg, alpha, l_max, mu_min, eps, "synthetic", s_nodes)
    assert ch[1][0] == oo
    assert ch[3][0] == O.cheby(n, ip, ix, dg, s, alpha, eps, False, katz=True, l_max=l_max, mu_min=mu_min,
                               sync=True)[2]
    sn, lt, gt = katz.solve_a_graph_gpu(n, ip, ix, dg, alpha, eps, s_nodes)
    assert (lt > 0).all() and (gt > 0).all()


def test_hk_functions(mods, cl):
    _, _, hk, _ = mods
    g, ip, ix, dg = cl
    n, tau, eps = g.n, 5.0, 1e-6
    s_nodes = graphs.uniform_seeds(g, 3, seed=9)
    s = int(s_nodes[0])
    assert hk.estimate_n(tau, eps) == O.hk_estimate_n(tau, eps)
    assert hk.estimate_coefficient(tau, 3) == pytest.approx(tau ** 4 / 24)
    est, x, _ = hk.hk_taylor_approx(n, ip, ix, dg, s, tau, eps)
    eo, xo = O.hk_taylor(n, ip, ix, dg, s, tau, eps)
    assert est == eo and np.abs(x - xo).sum() < 1e-10
    for local in (True, False):
        est, x, r, oper, beta_t, run_time, algo_time = hk.hk_sor_queue(n, ip, ix, dg, s, tau, eps, 1.0, local)
        eo, xo, ro, oo = O.hk_sor_queue(n, ip, ix, dg, s, tau, eps, 1.0, local)
        assert est == eo and oper == oo and np.abs(x - xo).sum() < 1e-10 and r.shape == (2, n)
    res = hk.solve_a_graph_all(n, ip, ix, dg, tau, eps, 1.2, "synthetic", s_nodes)
    assert len(res) == 13
    for j, sj in enumerate(s_nodes):
        assert res[5][j] == O.hk_sor_queue(n, ip, ix, dg, int(sj), tau, eps, 1.0, True)[3]
        assert res[3][j] == O.hk_sor_queue(n, ip, ix, dg, int(sj), tau, eps, 1.2, False)[3]
    opers, times, pk, ests = hk.solve_a_graph_pk(n, ip, ix, dg, tau, eps, 1.2, "synthetic", s_nodes)
    eo, xo, _, oo = O.hk_sor_queue(n, ip, ix, dg, s, tau, eps, 1.0, False)
    x1 = xo * n
    assert opers[0] == oo and ests[0] == O.hk_estimate_n(tau, .5 * eps)
    assert pk[0] == pytest.approx(((x1 ** 2).sum() ** 2) / (x1 ** 4).sum(), rel=1e-9)


def test_instantgnn_functions(mods):
    _, _, _, ign = mods
    g = graphs.chung_lu(2000, 2.2, 6.0, 100.0, seed=19)
    ip, ix, dg = _padded(g, 32)
    n, F, beta, eps = g.n, 4, 0.5, 1e-5
    X = np.random.default_rng(1).standard_normal((n, F))
    # static push of every column vs the synchronous oracle
    P, R = np.zeros((n, F)), X.copy()
    ign.instantGNNParallel(n, ip, ix, dg, ALPHA, eps, P, R, beta)
    Po, Ro = np.zeros((n, F)), X.copy()
    O.ign_sync(n, ip, ix, dg, ALPHA, eps, beta, Po, Ro)
    np.testing.assert_allclose(P, Po, rtol=1e-9, atol=1e-13)
    # one column from its queue, as instantGNNParallel builds it (InstantGNN.py:53-64)
    eps_vec = np.power(dg.astype(np.float64), 1 - beta) * eps
    r = X[:, 0].copy()
    p = np.zeros(n)
    act = np.flatnonzero(np.abs(r) >= eps_vec)
    queue = np.zeros(n + 2, np.int64)
    queue[1:1 + act.size] = act
    ign.instantGNNPush(n + 2, ip, ix, dg, ALPHA, eps_vec, p, r, queue, 0, act.size, np.zeros(n), beta)
    np.testing.assert_allclose(p, Po[:, 0], rtol=1e-9, atol=1e-13)
    # relaxed push of one column vs the multicolour oracle
    col = O._padded_colors(ip, ix, dg)
    r = X[:, 1].copy()
    p = np.zeros(n)
    act = np.flatnonzero(np.abs(r) >= eps_vec)
    queue[:] = 0
    queue[1:1 + act.size] = act
    ign.instantGNNSorPush(n + 2, ip, ix, dg, ALPHA, eps_vec, 1.2, p, r, queue, 0, act.size, np.zeros(n), beta)
    Ps, Rs = np.zeros((n, 1)), X[:, 1:2].copy()
    cand = np.zeros(n, np.uint8)
    cand[act] = 1
    O.ign_sor_color(n, ip, ix, dg, ALPHA, eps, beta, 1.2, Ps, Rs, col, cand0=cand)
    np.testing.assert_allclose(p, Ps[:, 0], rtol=1e-9, atol=1e-13)
    # the snapshot update, batched and per column
    us, vs = _mixed_batch(g, 100, 100, 20, seed=7)
    for algo in ("fwd", "insert-fwd"):
        ixa, dga = ix.copy(), dg.copy()
        Pb, Rb = P.copy(), R.copy()
        ign.instantGNNUpdateBatchParallel(n, ip, ixa, dga, ALPHA, eps, 1.0, Pb, Rb, X, us, vs, beta, algo)
        ixo, dgo = ix.copy(), dg.copy()
        Po2, Ro2 = P.copy(), R.copy()
        O.ign_update(n, ip, ixo, dgo, ALPHA, eps, 1.0, Po2, Ro2, X, us, vs, beta, algo, sync=True)
        np.testing.assert_array_equal(ixa, ixo)
        np.testing.assert_allclose(Pb, Po2, rtol=1e-9, atol=1e-13)
        # updetaGraph + instantGNNUpdateBatch, column by column
        ixc, dgc = ix.copy(), dg.copy()
        old = dgc.copy()
        ins, dele = ign.updetaGraph(ip, ixc, dgc, us, vs, onlyinsert="insert" in algo)
        np.testing.assert_array_equal(ixc, ixo)
        ev = np.power(dgc.astype(np.float64), 1 - beta) * eps
        for f in range(F):
            p, r = P[:, f].copy(), R[:, f].copy()
            ign.instantGNNUpdateBatch(n, ip, ixc, dgc, old, p, r, X[:, f].copy(), ALPHA, np.zeros(n + 2, np.int64), 0,
                                      0, np.zeros(n), ev, ins, dele, algo=algo, omega=1.0, beta=beta)
            np.testing.assert_allclose(p, Po2[:, f], rtol=1e-9, atol=1e-13)
            np.testing.assert_allclose(r, Ro2[:, f], rtol=1e-9, atol=1e-13)


def _save_npz(tmp_path, name, g):
    import scipy.sparse as sp
    d = tmp_path / "dataset" / name
    d.mkdir(parents=True)
    A = sp.csr_matrix((np.ones(g.indices.shape[0]), g.indices, g.indptr), shape=(g.n, g.n))
    sp.save_npz(d / f"{name}_csr-mat.npz", A)
    return str(tmp_path / "dataset") + "/"


def test_demo_call_sequence(mods, tmp_path):
    """demo.py:17-56's steps: load the CSR, float degree from adj.sum(1), optimal omega, then the three drivers."""
    import scipy.sparse as sp
    from ppr_solver import solve_a_graph_all, solve_a_graph_cheby, solve_a_graph_gpu
    path = _save_npz(tmp_path, "synthetic", graphs.chung_lu(3000, 2.1, 8.0, 300.0, seed=29))
    np.random.seed(17)
    alpha, eps, test_num = 0.2, 1e-5, 8
    alpha = alpha / (2 - alpha)
    mu = (1. - alpha) / (1. + alpha)
    omega = 1. + (mu / (1. + np.sqrt(1. - mu ** 2.))) ** 2.
    alpha = 2 * alpha / (1 + alpha)
    adj_matrix = sp.load_npz(path + "synthetic/synthetic_csr-mat.npz")
    indices, indptr = adj_matrix.indices, adj_matrix.indptr
    n = len(indptr) - 1
    degree = np.array(adj_matrix.sum(1)).flatten()
    s_nodes = np.random.randint(n, size=test_num)
    s_nodes = np.array(list(np.unique(s_nodes).astype(np.int32)))
    graph_result = solve_a_graph_all(n, indptr, indices, degree, alpha, eps, omega, "synthetic", s_nodes)
    cheby_result = solve_a_graph_cheby(n, indptr, indices, degree, alpha, eps, omega, "synthetic", s_nodes)
    gpu_result = solve_a_graph_gpu(n, indptr, indices, degree, alpha, eps, s_nodes)
    for i in range(12):
        assert np.isfinite(graph_result[i + 1].mean())
    for i in range(4):
        assert np.isfinite(cheby_result[i + 1].mean())
    for i in range(2):
        assert gpu_result[i + 1].mean() > 0
    for j, s in enumerate(s_nodes):
        assert graph_result[9][j] == O.ppr_gd(n, indptr, indices, degree, int(s), alpha, eps, True)[2]


def test_epsilon_sweep_call_sequence(mods, tmp_path):
    """test_epsilon.py:36-50's loop: eps from 2^8/n halving, skipping eps >= 1/d_max, solve_a_graph_all each."""
    import scipy.sparse as sp
    from ppr_solver import optimal_omega, solve_a_graph_all
    path = _save_npz(tmp_path, "synthetic", graphs.chung_lu(2000, 2.1, 8.0, 200.0, seed=31))
    adj_matrix = sp.load_npz(path + "synthetic/synthetic_csr-mat.npz")
    indices, indptr = adj_matrix.indices, adj_matrix.indptr
    n = len(indptr) - 1
    degree = np.array(adj_matrix.sum(1)).flatten()
    alpha, omega = optimal_omega(0.2)
    s_nodes = np.array(list(np.unique(np.random.default_rng(3).integers(n, size=6)).astype(np.int32)))
    eps = np.power(2.0, 8) / n
    results = {}
    while len(results) < 3:
        if eps >= 1 / degree.max():
            eps /= 2
            continue
        results[eps] = solve_a_graph_all(n, indptr, indices, degree, alpha, eps, omega, "synthetic", s_nodes)
        eps /= 2
    opers = [r[9].mean() for r in results.values()]
    assert opers[0] <= opers[1] <= opers[2] and opers[0] < opers[2]  # smaller eps, more work
