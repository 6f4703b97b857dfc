"""GPU parity: the CUDA engine (through the C ABI) against the oracle.

FP64 runs must reproduce the oracle's operation counts exactly (the frontier
sets are the reference's; only the order of atomic additions differs) and
its solutions to 1e-12 relative l1.  FP32 runs (FP32 residuals, Kahan FP32
solution, FP64 threshold tests) must stay within the stated l1 tolerance.
"""
import numpy as np
import pytest

import golden_cases as G
from gde import _lib as L
from gde import api, graphs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_L1 = 1e-12      # relative l1 of FP64 solutions vs the oracle
FP32_L1 = 2e-6       # mean relative l1 of FP32 solutions vs the FP64 oracle
OPER_RTOL = 1e-12


def fp32_flip_bound(g, eps, alpha):
    """Largest relative l1 an FP32 solve may show against the FP64 oracle.

    FP32 residual rounding can move a node whose FP64 residual lies within
    rounding of its threshold eps*alpha*d_u to the other side; the node then
    pushes a round earlier or later (or, at the end, not at all), which moves
    about 2*eps*alpha*d_u of mass in l1 (sum(x) ~ 1).  Allow a few such flips
    at the largest degree on top of the rounding error itself.
    """
    return FP32_L1 + 3 * 2 * eps * alpha * float(g.degree.max())


@pytest.fixture(scope="module")
def cl():
    g = graphs.chung_lu(3000, 2.1, 8.0, 300.0, seed=3)
    return g, api.Graph(g.indptr, g.indices)


@pytest.fixture(scope="module")
def golden_graphs():
    out = {}
    for name, d in G.graphs().items():
        out[name] = (d, api.Graph(d["indptr"], d["indices"]))
    return out


def rel_l1(a, b):
    return np.abs(np.asarray(a, np.float64) - b).sum() / max(np.abs(b).sum(), 1e-300)


@pytest.mark.parametrize("W", [1, 4, 8])
@pytest.mark.parametrize("local", [True, False])
def test_ppr_gd_fp64_matches_oracle(cl, W, local):
    g, Gd = cl
    deg = g.degree.astype(np.float64)
    seeds = graphs.uniform_seeds(g, 6, seed=7)
    eps = np.array([1e-4, 1e-5, 1e-6, 3e-6, 1e-5, 2e-7])
    res = api.solve(Gd, L.PPR, L.LOCAL_GD if local else L.GLOBAL_GD, seeds, eps, prec="fp64", alpha=0.15, tile_w=W)
    for i, s in enumerate(seeds):
        xo, ro, oo = O.ppr_gd(g.n, g.indptr, g.indices, deg, int(s), 0.15, eps[i], local)
        assert res["oper"][i] == pytest.approx(oo, rel=OPER_RTOL), (i, res["oper"][i], oo)
        assert rel_l1(res["x"][i], xo) < FP64_L1
        assert np.abs(res["r"][i] - ro).sum() < 1e-12


@pytest.mark.parametrize("W", [1, 8, 32])
def test_ppr_gd_fp32_within_tolerance(cl, W):
    g, Gd = cl
    deg = g.degree.astype(np.float64)
    seeds = graphs.uniform_seeds(g, 12, seed=8)
    eps = 1e-6
    res = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, eps, prec="fp32", alpha=0.1, tile_w=W)
    assert res["x"].dtype == np.float32
    errs = []
    for i, s in enumerate(seeds):
        xo, _, oo = O.ppr_gd(g.n, g.indptr, g.indices, deg, int(s), 0.1, eps, True)
        errs.append(rel_l1(res["x"][i], xo))
        assert errs[-1] < fp32_flip_bound(g, eps, 0.1), (i, errs[-1])
        # FP32 residuals can flip a threshold tie: opers agree to a few edges
        assert abs(res["oper"][i] - oo) <= 1e-3 * oo
    assert np.mean(errs) < FP32_L1, errs


def test_ppr_gd_against_reference_golden(golden_graphs):
    for c in G.cases("ppr_gd"):
        d, Gd = golden_graphs[c["graph"]]
        p = c["p"]
        res = api.solve(Gd, L.PPR, L.LOCAL_GD if p["local"] else L.GLOBAL_GD, [int(p["s"])], [p["eps"]],
                        prec="fp64", alpha=p["alpha"])
        assert res["oper"][0] == int(c["o"]["oper"]), c["id"]
        assert rel_l1(res["x"][0], c["o"]["x"]) < FP64_L1, c["id"]


@pytest.mark.parametrize("local", [True, False])
def test_katz_gd_fp64(golden_graphs, local):
    for c in G.cases("katz_gd"):
        if bool(c["p"]["local"]) != local:
            continue
        d, Gd = golden_graphs[c["graph"]]
        p = c["p"]
        res = api.solve(Gd, L.KATZ, L.LOCAL_GD if local else L.GLOBAL_GD, [int(p["s"])], [p["eps"]], prec="fp64",
                        alpha=p["alpha"])
        assert res["oper"][0] == int(c["o"]["oper"]), c["id"]
        assert rel_l1(res["x"][0], c["o"]["x"]) < 1e-11, c["id"]


@pytest.mark.parametrize("local", [True, False])
def test_ppr_cheby_fp64_sync_rule(golden_graphs, local):
    for c in G.cases("ppr_cheby"):
        if bool(c["p"]["local"]) != local:
            continue
        d, Gd = golden_graphs[c["graph"]]
        p = c["p"]
        n = len(d["indptr"]) - 1
        deg = np.diff(d["indptr"]).astype(np.float64)
        xo, ro, oo = O.cheby(n, d["indptr"], d["indices"], deg, int(p["s"]), p["alpha"], p["eps"], local, sync=True)
        res = api.solve(Gd, L.PPR, L.LOCAL_CHEBY if local else L.GLOBAL_CHEBY, [int(p["s"])], [p["eps"]],
                        prec="fp64", alpha=p["alpha"])
        assert res["oper"][0] == pytest.approx(oo, rel=OPER_RTOL), c["id"]
        assert rel_l1(res["x"][0], xo) < 1e-11, c["id"]
        # the reference's own (sequential-sweep) answer is an eps-solution too
        assert np.abs(res["x"][0] - c["o"]["x"]).sum() < 50 * p["eps"] * deg.sum(), c["id"]


def test_katz_cheby_fp64_sync_rule(golden_graphs):
    for c in G.cases("katz_cheby"):
        d, Gd = golden_graphs[c["graph"]]
        p = c["p"]
        n = len(d["indptr"]) - 1
        deg = np.diff(d["indptr"]).astype(np.float64)
        local = bool(p["local"])
        xo, ro, oo = O.cheby(n, d["indptr"], d["indices"], deg, int(p["s"]), p["alpha"], p["eps"], local, katz=True,
                             l_max=p["l_max"], mu_min=p["mu_min"], sync=True)
        res = api.solve(Gd, L.KATZ, L.LOCAL_CHEBY if local else L.GLOBAL_CHEBY, [int(p["s"])], [p["eps"]],
                        prec="fp64", alpha=p["alpha"], l_max=p["l_max"], mu_min=p["mu_min"])
        assert res["oper"][0] == pytest.approx(oo, rel=OPER_RTOL), c["id"]
        assert rel_l1(res["x"][0], xo) < 1e-10, c["id"]


def test_hk_level_push_matches_reference(golden_graphs):
    for c in G.cases("hk_sor_queue"):
        p = c["p"]
        if p["omega"] != 1.0:
            continue
        d, Gd = golden_graphs[c["graph"]]
        local = bool(p["local"])
        res = api.solve(Gd, L.HK, L.HK_LOCAL if local else L.HK_GLOBAL, [int(p["s"])], [p["eps"]], prec="fp64",
                        tau=p["tau"])
        assert res["oper"][0] == pytest.approx(float(c["o"]["oper"]), rel=OPER_RTOL), c["id"]
        assert rel_l1(res["x"][0], c["o"]["x"]) < 1e-11, c["id"]
        np.testing.assert_allclose(res["r"][0], c["o"]["r"], rtol=1e-9, atol=1e-15)


@pytest.mark.parametrize("omega", [0.8, 1.3, 1.6])
@pytest.mark.parametrize("local", [True, False])
def test_hk_relaxed_level_push_matches_oracle(golden_graphs, omega, local):
    """HK with relaxation omega != 1: the level-synchronous oracle (which is the reference's
    own result for the global sweeps) gives the same opers and solution."""
    seen = set()
    for c in G.cases("hk_sor_queue"):
        p = c["p"]
        key = (c["graph"], int(p["s"]), float(p["tau"]), float(p["eps"]))
        if key in seen:
            continue
        seen.add(key)
        d, Gd = golden_graphs[c["graph"]]
        n = len(d["indptr"]) - 1
        deg = np.diff(d["indptr"]).astype(np.float64)
        _, xo, _, oo = O.hk_sor_queue(n, d["indptr"], d["indices"], deg, int(p["s"]), p["tau"], p["eps"], omega, local,
                                      sync=True)
        res = api.solve(Gd, L.HK, L.HK_LOCAL if local else L.HK_GLOBAL, [int(p["s"])], [p["eps"]], prec="fp64",
                        tau=p["tau"], omega=omega)
        assert res["oper"][0] == pytest.approx(oo, rel=OPER_RTOL), c["id"]
        assert rel_l1(res["x"][0], xo) < 1e-11, c["id"]


def test_hk_omega_outside_the_convergent_range_is_rejected(golden_graphs):
    d, Gd = next(iter(golden_graphs.values()))
    for omega in (2.0, -0.5):
        with pytest.raises(L.GDEError) as ei:
            api.solve(Gd, L.HK, L.HK_LOCAL, [0], [1e-5], prec="fp64", tau=3.0, omega=omega)
        assert ei.value.status == L.GDE_EINVAL


def test_hk_taylor_matches_reference(golden_graphs):
    for c in G.cases("hk_taylor_approx"):
        p = c["p"]
        d, Gd = golden_graphs[c["graph"]]
        res = api.solve(Gd, L.HK, L.HK_TAYLOR, [int(p["s"])], [p["eps"]], prec="fp64", tau=p["tau"], want_r=False)
        assert rel_l1(res["x"][0], c["o"]["x"]) < 1e-11, c["id"]


def test_batched_mixed_eps_columns_are_independent(cl):
    """A query's answer is the same alone and inside a tile of other queries."""
    g, Gd = cl
    seeds = graphs.uniform_seeds(g, 16, seed=11)
    rng = np.random.default_rng(2)
    eps = np.exp(rng.uniform(np.log(1e-7), np.log(1e-5), 16))
    both = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, eps, prec="fp64", alpha=0.1, tile_w=8)
    for i in (0, 5, 13):
        alone = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds[i:i + 1], eps[i:i + 1], prec="fp64", alpha=0.1, tile_w=1)
        assert alone["oper"][0] == pytest.approx(both["oper"][i], rel=OPER_RTOL)
        assert rel_l1(both["x"][i], alone["x"][0]) < FP64_L1


def test_plain_baseline_close_to_oracle(cl):
    import torch
    g, Gd = cl
    deg = g.degree.astype(np.float64)
    s = int(graphs.uniform_seeds(g, 1, seed=3)[0])
    x = torch.zeros(g.n, dtype=torch.float32, device="cuda")
    oper, rounds = api.plain_ppr_local(Gd, s, 0.1, 1e-6, x_out=x)
    xo, _, oo = O.ppr_gd(g.n, g.indptr, g.indices, deg, s, 0.1, 1e-6, True)
    assert rel_l1(x.cpu().numpy(), xo) < 1e-4
    assert abs(oper - oo) <= 1e-2 * oo


def test_instantgnn_static_sync_oracle():
    dy = G.dyn()
    n = len(dy["indptr"]) - 1
    import torch
    X = dy["X"]
    alpha, eps, beta = 0.1, 1e-4, 0.5
    Gd = api.Graph(dy["indptr"], dy["indices"], row_len=dy["degree"], degree=dy["degree"].astype(np.float64))
    Po = np.zeros_like(X)
    Ro = X.copy()
    oo = O.ign_sync(n, dy["indptr"], dy["indices"], dy["degree"], alpha, eps, beta, Po, Ro)
    P = torch.zeros(X.shape, dtype=torch.float64, device="cuda")
    R = torch.from_numpy(X.copy()).cuda()
    res = api.feature_push(Gd, L.IGN, P, R, eps, alpha=alpha, beta=beta, prec="fp64", tile_w=2)
    np.testing.assert_allclose(res["oper"], oo, rtol=OPER_RTOL)
    np.testing.assert_allclose(P.cpu().numpy(), Po, rtol=1e-9, atol=1e-13)
    np.testing.assert_allclose(R.cpu().numpy(), Ro, rtol=1e-9, atol=1e-13)
    # the reference's FIFO push reaches an eps-solution of the same system
    st = [c for c in G.cases("instantgnn_static") if str(c["p"]["algo"]) == "fwdbatchinsert"][0]
    assert np.abs(P.cpu().numpy() - st["o"]["P"]).max() < 50 * eps * dy["degree"].max()


@pytest.mark.parametrize("algo", ["fwdbatchinsert", "fwdbatch"])
def test_instantgnn_update_matches_sync_oracle(algo):
    import torch
    dy = G.dyn()
    n = len(dy["indptr"]) - 1
    X = dy["X"]
    alpha, eps, beta = 0.1, 1e-4, 0.5
    ip = dy["indptr"].copy()
    ix_o = dy["indices"].astype(np.int32).copy()
    dg_o = dy["degree"].astype(np.int64).copy()
    ix = ix_o.copy()
    dg = dg_o.copy()
    Po = np.zeros_like(X)
    Ro = X.copy()
    O.ign_sync(n, ip, ix_o, dg_o, alpha, eps, beta, Po, Ro)
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    P = torch.zeros(X.shape, dtype=torch.float64, device="cuda")
    R = torch.from_numpy(X.copy()).cuda()
    Xd = torch.from_numpy(X.copy()).cuda()
    api.feature_push(Gd, L.IGN, P, R, eps, alpha=alpha, beta=beta, prec="fp64")
    updates = sorted([c for c in G.cases("instantgnn_update") if str(c["p"]["algo"]) == algo],
                     key=lambda c: int(c["p"]["snap"]))
    for c in updates:
        us, vs = c["o"]["us"], c["o"]["vs"]
        _, oo = O.ign_update(n, ip, ix_o, dg_o, alpha, eps, 1.0, Po, Ro, X, us, vs, beta, algo, sync=True)
        res = api.feature_update(Gd, L.IGN, ix, dg, us, vs, "insert" in algo, P, R, Xd, eps, alpha=alpha, beta=beta,
                                 prec="fp64")
        # the graph edit is bit-exact with the reference's own arrays
        np.testing.assert_array_equal(ix, c["o"]["indices"])
        np.testing.assert_array_equal(dg, c["o"]["degree"])
        np.testing.assert_allclose(res["oper"], oo, rtol=OPER_RTOL)
        np.testing.assert_allclose(P.cpu().numpy(), Po, rtol=1e-9, atol=1e-13)
        np.testing.assert_allclose(R.cpu().numpy(), Ro, rtol=1e-9, atol=1e-13)


def test_update_ppr_matches_sync_oracle():
    import torch
    dy = G.dyn()
    n = len(dy["indptr"]) - 1
    seeds = G.load()["dynppr/seeds"]
    alpha, eps = 0.1, 1e-4
    ip = dy["indptr"].copy()
    ix_o = dy["indices"].astype(np.int32).copy()
    dg_o = dy["degree"].astype(np.int64).copy()
    ix, dg = ix_o.copy(), dg_o.copy()
    Po = np.zeros((len(seeds), n))
    Ro = np.zeros((len(seeds), n))
    for f, s in enumerate(seeds):
        Ro[f, s] = alpha
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    P = torch.zeros((n, len(seeds)), dtype=torch.float64, device="cuda")
    R = torch.from_numpy(np.ascontiguousarray(Ro.T)).cuda()
    for snap in range(2):
        oo = O.update_ppr(n, ip, ix_o, dg_o, alpha, eps, 1.0, Po, Ro, dy["Us"][snap], dy["Vs"][snap], sync=True)
        res = api.feature_update(Gd, L.UPPR, ix, dg, dy["Us"][snap], dy["Vs"][snap], False, P, R, None, eps,
                                 alpha=alpha, prec="fp64", tile_w=1)
        np.testing.assert_array_equal(ix, ix_o)
        np.testing.assert_array_equal(dg, dg_o)
        np.testing.assert_allclose(res["oper"], oo, rtol=OPER_RTOL)
        np.testing.assert_allclose(P.cpu().numpy().T, Po, rtol=1e-9, atol=1e-13)
        np.testing.assert_allclose(R.cpu().numpy().T, Ro, rtol=1e-9, atol=1e-13)
