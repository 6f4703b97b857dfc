"""GPU LocalSOR / global SOR (multicolour order) against the oracle's restatement.

``oracle.sor_color`` runs the same multicolour Gauss-Seidel order
sequentially on the CPU in FP64, given the colouring the GPU uses; the GPU
must reproduce its operation counts and sweeps exactly and its solution to
1e-12 (only the order of additions at a target differs).  The colouring is
a proper colouring and equals greedy colouring in degree-descending order.
"""
import numpy as np
import pytest

from gde import _lib as L
from gde import api, graphs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_L1 = 1e-12


@pytest.fixture(scope="module")
def cl():
    g = graphs.chung_lu(3000, 2.1, 8.0, 300.0, seed=3)
    return g, api.Graph(g.indptr, g.indices)


def rel_l1(a, b):
    return np.abs(np.asarray(a, np.float64) - b).sum() / max(np.abs(b).sum(), 1e-300)


def test_colouring_is_proper_and_greedy(cl):
    g, Gd = cl
    col = api.graph_colors(Gd)
    src = np.repeat(np.arange(g.n), np.diff(g.indptr))
    assert (col[src] != col[g.indices]).all()
    order = np.argsort(-np.diff(g.indptr), kind="stable")
    np.testing.assert_array_equal(col, O.greedy_colors(g.indptr, g.indices, order))


@pytest.mark.parametrize("omega", [1.0, 1.3, 1.7])
@pytest.mark.parametrize("local", [True, False])
def test_ppr_sor_fp64_matches_oracle(cl, omega, local):
    g, Gd = cl
    deg = g.degree.astype(np.float64)
    col = api.graph_colors(Gd)
    seeds = graphs.uniform_seeds(g, 4, seed=12)
    eps = 1e-6 if local else 1e-5
    res = api.sor(Gd, L.PPR, seeds, eps, omega=omega, local=local, alpha=0.1)
    for i, s in enumerate(seeds):
        xo, ro, oo, so = O.sor_color(g.n, g.indptr, g.indices, deg, int(s), 0.1, eps, omega, local, col)
        assert res["oper"][i] == pytest.approx(oo, rel=1e-12), (i, res["oper"][i], oo)
        assert res["sweeps"][i] == so
        assert rel_l1(res["x"][i], xo) < FP64_L1
        assert np.abs(res["r"][i] - ro).sum() < 1e-12


def test_katz_sor_fp64_matches_oracle(cl):
    g, Gd = cl
    deg = g.degree.astype(np.float64)
    col = api.graph_colors(Gd)
    alpha = 1.0 / (float(g.degree.max()) + 1.0)
    seeds = graphs.uniform_seeds(g, 3, seed=13)
    res = api.sor(Gd, L.KATZ, seeds, 1e-6, omega=1.2, local=True, alpha=alpha)
    for i, s in enumerate(seeds):
        xo, _, oo, so = O.sor_color(g.n, g.indptr, g.indices, deg, int(s), alpha, 1e-6, 1.2, True, col, katz=True)
        assert res["oper"][i] == pytest.approx(oo, rel=1e-12)
        assert rel_l1(res["x"][i], xo) < FP64_L1


def test_sor_converges_like_the_reference_order(cl):
    """Multicolour order vs the reference's FIFO order: same stopping rule, similar work and error."""
    g, Gd = cl
    deg = g.degree.astype(np.float64)
    s = int(graphs.uniform_seeds(g, 1, seed=14)[0])
    truth = O.global_solve_ppr(g.indptr, g.indices, deg, s, 0.1)
    res = api.sor(Gd, L.PPR, [s], 1e-6, omega=1.3, local=True, alpha=0.1)
    xf, _, of = O.sor(g.n, g.indptr, g.indices, deg, s, 0.1, 1e-6, 1.3, True)
    err_gpu = np.abs(res["x"][0] - truth).sum()
    err_fifo = np.abs(xf - truth).sum()
    assert err_gpu < 2 * err_fifo + 1e-9
    assert 0.5 * of < res["oper"][0] < 2 * of
    # every residual is below its threshold at the end
    assert (np.abs(res["r"][0]) < 1e-6 * 0.1 * deg).all()


def test_sor_batched_equals_single(cl):
    g, Gd = cl
    seeds = graphs.uniform_seeds(g, 6, seed=15)
    eps = np.array([1e-5, 1e-6, 3e-6, 1e-5, 2e-6, 1e-6])
    both = api.sor(Gd, L.PPR, seeds, eps, omega=1.4, local=True, alpha=0.1)
    for i in (0, 3, 5):
        one = api.sor(Gd, L.PPR, seeds[i:i + 1], eps[i:i + 1], omega=1.4, local=True, alpha=0.1)
        assert one["oper"][0] == pytest.approx(both["oper"][i], rel=1e-12)
        assert rel_l1(both["x"][i], one["x"][0]) < FP64_L1


def test_sor_fp32(cl):
    g, Gd = cl
    deg = g.degree.astype(np.float64)
    col = api.graph_colors(Gd)
    seeds = graphs.uniform_seeds(g, 6, seed=16)
    res = api.sor(Gd, L.PPR, seeds, 1e-6, omega=1.3, local=True, alpha=0.1, prec="fp32")
    errs = []
    for i, s in enumerate(seeds):
        xo, _, oo, _ = O.sor_color(g.n, g.indptr, g.indices, deg, int(s), 0.1, 1e-6, 1.3, True, col)
        errs.append(rel_l1(res["x"][i], xo))
        assert errs[-1] < 2e-6 + 6 * 1e-7 * float(g.degree.max())
        assert abs(res["oper"][i] - oo) <= 1e-2 * oo
    assert np.mean(errs) < 1e-5


def _dyn():
    import golden_cases as G
    return G.dyn(), G


def test_instantgnn_sor_static_matches_oracle():
    import torch
    dy, _ = _dyn()
    n = len(dy["indptr"]) - 1
    X = dy["X"]
    alpha, eps, beta, omega = 0.1, 1e-4, 0.5, 1.3
    ip = dy["indptr"].copy()
    ix = dy["indices"].astype(np.int32).copy()
    dg = dy["degree"].astype(np.int64).copy()
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    col = api.graph_colors(Gd)
    Po = np.zeros_like(X)
    Ro = X.copy()
    oo = O.ign_sor_color(n, ip, ix, dg, alpha, eps, beta, omega, Po, Ro, col)
    P = torch.zeros(X.shape, dtype=torch.float64, device="cuda")
    R = torch.from_numpy(X.copy()).cuda()
    res = api.feature_push(Gd, L.IGN, P, R, eps, alpha=alpha, beta=beta, prec="fp64", omega=omega)
    np.testing.assert_allclose(res["oper"], oo, rtol=1e-12)
    np.testing.assert_allclose(P.cpu().numpy(), Po, rtol=1e-9, atol=1e-13)
    np.testing.assert_allclose(R.cpu().numpy(), Ro, rtol=1e-9, atol=1e-13)


def _padded(dy):
    ip = dy["indptr"].copy()
    ix = dy["indices"].astype(np.int32).copy()
    dg = dy["degree"].astype(np.int64).copy()
    return ip, ix, dg


def test_instantgnn_sor_update_matches_oracle():
    """Insert batches + repair + SOR push: exact against the oracle in the same colour order."""
    import torch
    dy, G = _dyn()
    n = len(dy["indptr"]) - 1
    X = dy["X"]
    alpha, eps, beta, omega = 0.1, 1e-4, 0.5, 1.25
    ip, ix, dg = _padded(dy)
    ix_o, dg_o = ix.copy(), dg.copy()
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    Po = np.zeros_like(X)
    Ro = X.copy()
    O.ign_sor_color(n, ip, ix_o, dg_o, alpha, eps, beta, omega, Po, Ro, api.graph_colors(Gd))
    P = torch.from_numpy(Po.copy()).cuda()
    R = torch.from_numpy(Ro.copy()).cuda()
    Xd = torch.from_numpy(X.copy()).cuda()
    for snap in range(3):
        us, vs = dy["Us"][snap], dy["Vs"][snap]
        _, oo = O.ign_update(n, ip, ix_o, dg_o, alpha, eps, omega, Po, Ro, X, us, vs, beta, "insert_sor", color=True)
        res = api.feature_update(Gd, L.IGN, ix, dg, us, vs, True, P, R, Xd, eps, alpha=alpha, beta=beta,
                                 prec="fp64", omega=omega)
        np.testing.assert_array_equal(ix, ix_o)
        np.testing.assert_array_equal(dg, dg_o)
        # the colouring follows the edited graph
        np.testing.assert_array_equal(api.graph_colors(Gd), O._padded_colors(ip, ix_o, dg_o))
        np.testing.assert_allclose(res["oper"], oo, rtol=1e-12)
        np.testing.assert_allclose(P.cpu().numpy(), Po, rtol=1e-9, atol=1e-13)
        np.testing.assert_allclose(R.cpu().numpy(), Ro, rtol=1e-9, atol=1e-13)


@pytest.mark.parametrize("omega", [1.2, 1.5])
def test_update_ppr_sor_matches_oracle(omega):
    """update_ppr_parallel with omega != 1 (insertions and deletions): exact in multicolour order."""
    import torch
    dy, G = _dyn()
    n = len(dy["indptr"]) - 1
    seeds = G.load()["dynppr/seeds"]
    alpha, eps = 0.1, 1e-5
    ip, ix, dg = _padded(dy)
    ix_o, dg_o = ix.copy(), dg.copy()
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    Po = np.zeros((len(seeds), n))
    Ro = np.zeros((len(seeds), n))
    for f, s in enumerate(seeds):
        Ro[f, s] = alpha
    P = torch.zeros((n, len(seeds)), dtype=torch.float64, device="cuda")
    R = torch.from_numpy(np.ascontiguousarray(Ro.T)).cuda()
    for snap in range(3):
        oo = O.update_ppr(n, ip, ix_o, dg_o, alpha, eps, omega, Po, Ro, dy["Us"][snap], dy["Vs"][snap], color=True)
        res = api.feature_update(Gd, L.UPPR, ix, dg, dy["Us"][snap], dy["Vs"][snap], False, P, R, None, eps,
                                 alpha=alpha, prec="fp64", omega=omega)
        np.testing.assert_array_equal(ix, ix_o)
        np.testing.assert_array_equal(dg, dg_o)
        np.testing.assert_allclose(res["oper"], oo, rtol=1e-12)
        np.testing.assert_allclose(P.cpu().numpy().T, Po, rtol=1e-9, atol=1e-13)
        np.testing.assert_allclose(R.cpu().numpy().T, Ro, rtol=1e-9, atol=1e-13)


def test_instantgnn_sor_update_meets_stopping_rule():
    import torch
    dy, _ = _dyn()
    X = dy["X"]
    alpha, eps, beta = 0.1, 1e-4, 0.5
    out = {}
    for omega in (1.0, 1.3):
        ip = dy["indptr"].copy()
        ix = dy["indices"].astype(np.int32).copy()
        dg = dy["degree"].astype(np.int64).copy()
        Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
        P = torch.zeros(X.shape, dtype=torch.float64, device="cuda")
        R = torch.from_numpy(X.copy()).cuda()
        Xd = torch.from_numpy(X.copy()).cuda()
        api.feature_push(Gd, L.IGN, P, R, eps, alpha=alpha, beta=beta, prec="fp64", omega=omega)
        for snap in range(2):
            api.feature_update(Gd, L.IGN, ix, dg, dy["Us"][snap], dy["Vs"][snap], True, P, R, Xd, eps, alpha=alpha,
                               beta=beta, prec="fp64", omega=omega)
        thr = eps * np.power(dg.astype(np.float64), 1 - beta)
        Rn = R.cpu().numpy()
        absorbing = dg == 0
        assert (np.abs(Rn[~absorbing]) < thr[~absorbing, None]).all()
        out[omega] = P.cpu().numpy()
    # both pushes approximate the same propagated features to within the eps-level residual
    assert np.abs(out[1.3] - out[1.0]).max() < 50 * eps
