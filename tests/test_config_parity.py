"""Parity at the benchmark configurations' own sizes, against the FP64 oracle.

C1: the 100k-node Chung-Lu graph (power-law exponent 2.1, mean degree 10,
    max 2,000), PPR local GD in FP64 at eps = 1e-6 over 50 seeds: operation
    counts equal to the oracle's exactly, solutions to 1e-12 relative l1; one
    seed against an FP64 global solve (l1 error and the largest D^-1
    residual, which the stopping rule bounds by eps * alpha).
C2: the 2.36M-node wiki-talk-shaped graph, served FP32 PPR local GD at
    eps = 1e-7 (the benchmarked path) over 32 seeds against the FP64 oracle:
    every seed l1 <= 1e-6 and the mean <= 3e-7.  A node whose FP64 residual
    lies within FP32 rounding of its threshold may push a round apart, which
    moves about 2 eps alpha d of l1; the highest-degree nodes, where that is
    largest, keep their residual in FP64.  The operation-count difference is
    reported.
C5: the 169k-node InstantGNN graph, two snapshots of 59,375 inserted edges
    on 8 feature columns: FP64 P, R and operation counts against the
    oracle's synchronous update per snapshot; FP32 within a stated bound.
C3: 64 seeds in the tuned 8-column node x seed tiles, eps log-uniform in
    [1e-8, 1e-5], FP32 against the FP64 oracle at each seed's eps.
FP32 global GD (ppr_gd_standard_gpu, katz_gd_standard_gpu) on the C1 graph.
"""
import numpy as np
import pytest

from gde import _lib as L
from gde import api, graphs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c1():
    g = graphs.chung_lu_100k()
    return g, api.Graph(g.indptr, g.indices)


def test_c1_fp64_local_gd_50_seeds_exact(c1):
    g, Gd = c1
    alpha, eps = 0.1, 1e-6
    deg = g.degree.astype(np.float64)
    seeds = graphs.uniform_seeds(g, 50, seed=1)
    res = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, eps, prec="fp64", alpha=alpha, tile_w=1)
    oo, xo = O.ppr_gd_many(g.n, g.indptr, g.indices, deg, seeds, alpha, eps, local=True, keep_x=True)
    np.testing.assert_array_equal(res["oper"].astype(np.int64), oo)
    rel = np.abs(res["x"] - xo).sum(1) / np.abs(xo).sum(1)
    assert rel.max() < 1e-12, rel.max()
    # one seed against the PPR vector itself (FP64 global solve to 1e-15)
    s = int(seeds[0])
    truth = O.global_solve_ppr(g.indptr, g.indices, deg, s, alpha)
    l1_gpu = np.abs(res["x"][0] - truth).sum()
    l1_oracle = np.abs(xo[0] - truth).sum()
    assert abs(l1_gpu - l1_oracle) < 1e-12
    assert np.max(np.abs(res["r"][0]) / deg) < eps * alpha
    # the local push leaves at most eps*alpha*vol of residual mass; l1 error is bounded by it / alpha
    assert l1_gpu <= eps * alpha * deg.sum() / alpha


def test_c1_fp32_global_gd_ppr_and_katz(c1):
    g, Gd = c1
    deg = g.degree.astype(np.float64)
    seeds = graphs.uniform_seeds(g, 4, seed=2)
    n, m = g.n, deg.sum()
    for kind, alpha, eps in ((L.PPR, 0.1, 1e-6), (L.KATZ, 0.5 / deg.max(), 1e-6)):
        res = api.solve(Gd, kind, L.GLOBAL_GD, seeds, eps, prec="fp32", alpha=alpha, tile_w=4)
        for i, s in enumerate(seeds):
            fn = O.ppr_gd if kind == L.PPR else O.katz_gd
            xo, _, oo = fn(n, g.indptr, g.indices, deg, int(s), alpha, eps, False)
            iters_o = round(oo / (n + m))
            iters = round(res["oper"][i] / (n + m))
            # FP32 residuals can move the last CHECK by one iteration
            assert abs(iters - iters_o) <= 1, (kind, i, iters, iters_o)
            err = np.abs(res["x"][i].astype(np.float64) - xo).sum() / np.abs(xo).sum()
            assert err < 1e-5, (kind, i, err)


def test_c3_node_seed_tiles_fp32_against_fp64_oracle(c1):
    """C3's tuned shape: 64 seeds in 8-column node x seed tiles (short rows up to 16 edges), eps
    log-uniform in [1e-8, 1e-5], FP32 residuals, against the FP64 oracle at each seed's eps.

    A node whose FP64 residual lies within FP32 rounding of its threshold eps alpha d pushes a
    round apart, which moves about 2 eps alpha d of l1.  Over a query's hundreds of rounds such
    ties recur: on this graph the worst seeds of both the tiles and the served slots show 3 to 5
    of them at the largest degree (relative l1 up to 2.6e-4 at eps 2.6e-7), most seeds none.  Each
    seed is held to 10 at the largest degree, the mean to 2e-5, operation counts to 0.1%."""
    g, Gd = c1
    alpha = 0.1
    deg = g.degree.astype(np.float64)
    rng = np.random.default_rng(2)
    seeds = graphs.uniform_seeds(g, 64, seed=3)
    eps = np.exp(rng.uniform(np.log(1e-8), np.log(1e-5), 64))
    res = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, eps, prec="fp32", alpha=alpha, tile_w=8,
                    tuning={"small_max": 16})
    rels = []
    for i, s in enumerate(seeds):
        xo, _, oo = O.ppr_gd(g.n, g.indptr, g.indices, deg, int(s), alpha, float(eps[i]), True)
        rel = np.abs(res["x"][i].astype(np.float64) - xo).sum() / np.abs(xo).sum()
        rels.append(rel)
        assert rel < 2e-6 + 10 * 2 * eps[i] * alpha * deg.max(), (i, eps[i], rel)
        assert abs(res["oper"][i] - oo) <= 1e-3 * oo, (i, res["oper"][i], oo)
    assert np.mean(rels) < 2e-5, np.mean(rels)


def test_c2_served_fp32_l1_per_seed_against_fp64_oracle():
    g = graphs.chung_lu_wikitalk_shape()
    Gd = api.Graph(g.indptr, g.indices)
    alpha, eps = 0.1, 1e-7
    deg = g.degree.astype(np.float64)
    seeds = graphs.uniform_seeds(g, 32, seed=515151)
    res = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, eps, prec="fp32", alpha=alpha, tile_w=1, want_r=False,
                    tuning={"slots": 32})
    oo, xo = O.ppr_gd_many(g.n, g.indptr, g.indices, deg, seeds, alpha, eps, local=True, keep_x=True)
    l1 = np.abs(res["x"].astype(np.float64) - xo).sum(1)
    od = np.abs(res["oper"] - oo) / oo
    print(f"C2 served FP32 vs FP64 oracle: l1 max {l1.max():.3e} mean {l1.mean():.3e}; "
          f"oper rel diff max {od.max():.3e} (abs {np.abs(res['oper'] - oo).max():.0f})")
    assert l1.mean() <= 3e-7, l1
    assert l1.max() <= 1e-6, l1
    assert od.max() < 1e-4, od
    Gd.free()


C5_F, C5_ALPHA, C5_BETA, C5_EPS = 8, 0.1, 0.5, 1e-7


@pytest.fixture(scope="module")
def c5():
    """The graph, features and the oracle's state after the initial push and after each of two snapshots."""
    base = graphs.chung_lu_arxiv_shape()
    dyn = graphs.dynamic_padded(base, 950_000, 16, seed=1)
    n = dyn.n
    X = np.random.default_rng(3).standard_normal((n, 128))[:, :C5_F].copy()
    ip = dyn.indptr.astype(np.int64)
    ix, dg = dyn.indices.copy(), dyn.degree.copy()
    Po, Ro = np.zeros((n, C5_F)), X.copy()
    O.ign_sync(n, ip, ix, dg, C5_ALPHA, C5_EPS, C5_BETA, Po, Ro)
    snaps = []
    for s in range(2):
        _, oo = O.ign_update(n, ip, ix, dg, C5_ALPHA, C5_EPS, 1.0, Po, Ro, X, dyn.Us[s], dyn.Vs[s], C5_BETA,
                             "fwd-insert", sync=True)
        snaps.append((ix.copy(), dg.copy(), Po.copy(), Ro.copy(), oo))
    return dyn, X, snaps


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_c5_two_snapshots_against_the_oracle(c5, prec):
    import torch
    dyn, X, snaps = c5
    n = dyn.n
    ip = dyn.indptr.astype(np.int64)
    ix_d, dg_d = dyn.indices.copy(), dyn.degree.copy()
    Gd = api.Graph(ip, ix_d, row_len=dg_d, degree=dg_d.astype(np.float64))
    dt = torch.float64 if prec == "fp64" else torch.float32
    Xd = torch.from_numpy(X).to("cuda", dt)
    Pd = torch.zeros_like(Xd)
    Rd = Xd.clone()
    api.feature_push(Gd, L.IGN, Pd, Rd, C5_EPS, alpha=C5_ALPHA, beta=C5_BETA, prec=prec)
    for s in range(2):
        ix_o, dg_o, Po, Ro, oo = snaps[s]
        res = api.feature_update(Gd, L.IGN, ix_d, dg_d, dyn.Us[s], dyn.Vs[s], True, Pd, Rd, Xd, C5_EPS,
                                 alpha=C5_ALPHA, beta=C5_BETA, prec=prec)
        np.testing.assert_array_equal(ix_d, ix_o)
        np.testing.assert_array_equal(dg_d, dg_o)
        P, R = Pd.double().cpu().numpy(), Rd.double().cpu().numpy()
        if prec == "fp64":
            np.testing.assert_allclose(res["oper"], oo, rtol=1e-12)
            np.testing.assert_allclose(P, Po, rtol=1e-9, atol=1e-13)
            np.testing.assert_allclose(R, Ro, rtol=1e-9, atol=1e-13)
        else:
            # FP32 residuals: per column, the l1 distance of P relative to the FP64 oracle's
            rel = np.abs(P - Po).sum(0) / np.abs(Po).sum(0)
            od = np.abs(res["oper"] - oo) / oo
            print(f"C5 snapshot {s} FP32: P rel l1 max {rel.max():.3e}, oper rel diff max {od.max():.3e}")
            assert rel.max() < 1e-5, rel
            assert od.max() < 1e-2, od
