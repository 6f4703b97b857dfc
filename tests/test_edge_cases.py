"""Edge cases of the C ABI and the drop-ins, on the GPU.

Empty query lists, isolated and boundary seeds, ragged tiles, immediate
stops, padded graphs with sentinel slack, and argument errors that must come
back as the documented status codes (the reference only asserts).
"""
import numpy as np
import pytest

from gde import _lib as L
from gde import api, graphs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cl():
    g = graphs.chung_lu(2000, 2.1, 6.0, 150.0, seed=9)
    return g, api.Graph(g.indptr, g.indices)


def test_no_queries(cl):
    g, Gd = cl
    res = api.solve(Gd, L.PPR, L.LOCAL_GD, np.zeros(0, np.int32), 1e-6, prec="fp64", alpha=0.1)
    assert res["x"].shape == (0, g.n) and res["oper"].shape == (0,)
    res = api.serve(Gd, L.PPR, np.zeros(0, np.int32), 1e-6, alpha=0.1)
    assert res["oper"].shape == (0,)


def test_isolated_seed_keeps_its_mass():
    # a graph with isolated nodes (kept): PPR from an isolated seed stops after one push
    g = graphs.chung_lu(500, 2.3, 3.0, 40.0, seed=1, drop_isolated=False)
    iso = np.nonzero(np.diff(g.indptr) == 0)[0]
    assert iso.size > 0
    Gd = api.Graph(g.indptr, g.indices)
    s = int(iso[0])
    res = api.solve(Gd, L.PPR, L.LOCAL_GD, [s], [1e-4], prec="fp64", alpha=0.1)
    xo, ro, oo = O.ppr_gd(g.n, g.indptr, g.indices, g.degree.astype(np.float64), s, 0.1, 1e-4, True)
    assert res["oper"][0] == oo == 0
    np.testing.assert_allclose(res["x"][0], xo, atol=1e-15)


def test_boundary_eps_times_degree_is_one(cl):
    g, Gd = cl
    s = int(np.argmax(g.degree))
    eps = 1.0 / float(g.degree[s])  # eps * degree[s] == 1 passes ppr_solver.py:213
    while eps * float(g.degree[s]) > 1.0:
        eps = np.nextafter(eps, 0.0)
    res = api.solve(Gd, L.PPR, L.LOCAL_GD, [s], [eps], prec="fp64", alpha=0.1)
    xo, _, oo = O.ppr_gd(g.n, g.indptr, g.indices, g.degree.astype(np.float64), s, 0.1, eps, True)
    assert res["oper"][0] == oo
    assert np.abs(res["x"][0] - xo).sum() < 1e-12


def test_eps_above_boundary_is_rejected(cl):
    g, Gd = cl
    s = int(np.argmax(g.degree))
    with pytest.raises(L.GDEError) as ei:
        api.solve(Gd, L.PPR, L.LOCAL_GD, [s], [2.0 / float(g.degree[s])], prec="fp64", alpha=0.1)
    assert ei.value.status == L.GDE_EINVAL


@pytest.mark.parametrize("bad", ["seed", "eps", "kind", "tile"])
def test_argument_errors(cl, bad):
    g, Gd = cl
    kw = dict(prec="fp64", alpha=0.1)
    with pytest.raises(L.GDEError) as ei:
        if bad == "seed":
            api.solve(Gd, L.PPR, L.LOCAL_GD, [g.n], [1e-6], **kw)
        elif bad == "eps":
            api.solve(Gd, L.PPR, L.LOCAL_GD, [0], [0.0], **kw)
        elif bad == "kind":
            api.solve(Gd, L.IGN, L.LOCAL_GD, [0], [1e-6], **kw)
        else:
            api.solve(Gd, L.PPR, L.GLOBAL_GD, [0, 1, 2], [1e-6], tile_w=3, **kw)
    assert ei.value.status == L.GDE_EINVAL
    assert L.load().gde_last_error(Gd.ctx.ptr)  # a message is set


@pytest.mark.parametrize("W", [2, 4, 8, 32])
def test_ragged_tiles(cl, W):
    """A query count that is not a multiple of the tile width leaves idle columns."""
    g, Gd = cl
    deg = g.degree.astype(np.float64)
    seeds = graphs.uniform_seeds(g, W + 3, seed=4)
    res = api.solve(Gd, L.PPR, L.GLOBAL_GD, seeds, 1e-5, prec="fp64", alpha=0.15, tile_w=W)
    for i in (0, W, W + 2):
        xo, _, oo = O.ppr_gd(g.n, g.indptr, g.indices, deg, int(seeds[i]), 0.15, 1e-5, False)
        assert res["oper"][i] == pytest.approx(oo, rel=1e-12)
        assert np.abs(res["x"][i] - xo).sum() < 1e-12 * max(np.abs(xo).sum(), 1)


def test_immediate_stop(cl):
    """eps so large that only the seed pushes once (or not at all)."""
    g, Gd = cl
    s = int(graphs.uniform_seeds(g, 1, seed=2)[0])
    eps = 0.99 / float(g.degree[s])
    res = api.solve(Gd, L.PPR, L.LOCAL_GD, [s], [eps], prec="fp32", alpha=0.1)
    xo, _, oo = O.ppr_gd(g.n, g.indptr, g.indices, g.degree.astype(np.float64), s, 0.1, eps, True)
    assert res["oper"][0] == oo


def test_padded_graph_with_sentinel_slack():
    """A padded CSR (row capacity > degree, slack filled with n) solves like its compact form."""
    g = graphs.chung_lu(800, 2.2, 6.0, 80.0, seed=6)
    n = g.n
    deg = np.diff(g.indptr)
    cap = deg + 3
    ip = np.zeros(n + 1, np.int64)
    np.cumsum(cap, out=ip[1:])
    ix = np.full(ip[-1], n, np.int32)
    for u in range(n):
        ix[ip[u]:ip[u] + deg[u]] = g.indices[g.indptr[u]:g.indptr[u + 1]]
    Gp = api.Graph(ip, ix, row_len=deg.astype(np.int64), degree=deg.astype(np.float64))
    Gc = api.Graph(g.indptr, g.indices)
    seeds = graphs.uniform_seeds(g, 3, seed=8)
    a = api.solve(Gp, L.PPR, L.LOCAL_GD, seeds, 1e-6, prec="fp64", alpha=0.1, tile_w=4)
    b = api.solve(Gc, L.PPR, L.LOCAL_GD, seeds, 1e-6, prec="fp64", alpha=0.1, tile_w=4)
    np.testing.assert_allclose(a["oper"], b["oper"], rtol=1e-12)
    np.testing.assert_allclose(a["x"], b["x"], rtol=0, atol=1e-15)


def test_device_outputs(cl):
    import torch
    g, Gd = cl
    seeds = graphs.uniform_seeds(g, 5, seed=3)
    x = torch.full((5, g.n), float("nan"), dtype=torch.float32, device="cuda")
    api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, 1e-6, prec="fp32", alpha=0.1, want_r=False, x_out=x, device_out=True)
    host = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, 1e-6, prec="fp32", alpha=0.1, want_r=False)
    xd = x.cpu().numpy()
    assert np.isfinite(xd).all()
    # same algorithm, FP32 atomics in a different order: a few threshold flips at most
    assert np.abs(xd - host["x"]).sum() / np.abs(host["x"]).sum() < 1e-4


def test_served_on_a_padded_graph_matches_compact():
    """Served FP32 and FP64 queries on an unrelabelled padded CSR (no permutation on the
    read-out) agree with the relabelled compact graph."""
    g = graphs.chung_lu(800, 2.2, 6.0, 80.0, seed=7)
    n = g.n
    deg = np.diff(g.indptr)
    cap = deg + 2
    ip = np.zeros(n + 1, np.int64)
    np.cumsum(cap, out=ip[1:])
    ix = np.full(ip[-1], n, np.int32)
    for u in range(n):
        ix[ip[u]:ip[u] + deg[u]] = g.indices[g.indptr[u]:g.indptr[u + 1]]
    Gp = api.Graph(ip, ix, row_len=deg.astype(np.int64), degree=deg.astype(np.float64))
    Gc = api.Graph(g.indptr, g.indices)
    seeds = graphs.uniform_seeds(g, 9, seed=11)
    for prec, tol in (("fp64", 1e-12), ("fp32", 1e-5)):
        a = api.serve(Gp, L.KATZ, seeds, 1e-6, alpha=1.0 / (float(deg.max()) + 1.0), prec=prec, slots=3)
        b = api.serve(Gc, L.KATZ, seeds, 1e-6, alpha=1.0 / (float(deg.max()) + 1.0), prec=prec, slots=3)
        for i in range(len(seeds)):
            xa, xb = a["x"][i].astype(np.float64), b["x"][i].astype(np.float64)
            assert np.abs(xa - xb).sum() <= tol * max(np.abs(xb).sum(), 1.0), (prec, i)


def test_tables_follow_edits_of_another_kind():
    """An InstantGNN push after a dynamic-PPR edit batch (insertions and deletions) on the same
    graph sees the edited degrees: it equals the push on a fresh upload of the edited arrays."""
    import torch
    import golden_cases as GC
    dy = GC.dyn()
    n = len(dy["indptr"]) - 1
    ip = dy["indptr"].copy()
    ix = dy["indices"].astype(np.int32).copy()
    dg = dy["degree"].astype(np.int64).copy()
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    X = dy["X"]
    alpha, eps, beta = 0.1, 1e-4, 0.5
    P = torch.zeros(X.shape, dtype=torch.float64, device="cuda")
    R = torch.from_numpy(X.copy()).cuda()
    api.feature_push(Gd, L.IGN, P, R, eps, alpha=alpha, beta=beta, prec="fp64")  # builds the beta tables
    Pu = torch.zeros((n, 2), dtype=torch.float64, device="cuda")
    Ru = torch.zeros((n, 2), dtype=torch.float64, device="cuda")
    api.feature_update(Gd, L.UPPR, ix, dg, dy["Us"][0], dy["Vs"][0], False, Pu, Ru, None, eps, alpha=alpha,
                       prec="fp64")
    assert not np.array_equal(dg, dy["degree"])  # the batch changed degrees
    fresh = api.Graph(ip, ix.copy(), row_len=dg.copy(), degree=dg.astype(np.float64))
    out = []
    for G in (Gd, fresh):
        P2 = torch.zeros(X.shape, dtype=torch.float64, device="cuda")
        R2 = torch.from_numpy(X.copy()).cuda()
        res = api.feature_push(G, L.IGN, P2, R2, eps, alpha=alpha, beta=beta, prec="fp64")
        out.append((res["oper"], P2.cpu().numpy()))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_allclose(out[0][1], out[1][1], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("kind", [L.IGN, L.UPPR])
def test_feature_push_one_column_tiles_match_wide_tiles(kind):
    """One-column tiles (flattened short-row scatter, target scaling per edge) give the
    same FP64 result as 8-column tiles."""
    import torch
    import golden_cases as GC
    dy = GC.dyn()
    ip = dy["indptr"].copy()
    ix = dy["indices"].astype(np.int32).copy()
    dg = dy["degree"].astype(np.int64).copy()
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    X = np.concatenate([dy["X"], dy["X"][:, :2] * 0.5], axis=1)  # 8 columns
    out = []
    for W in (1, 8):
        P = torch.zeros(X.shape, dtype=torch.float64, device="cuda")
        R = torch.from_numpy(np.ascontiguousarray(X)).cuda()
        res = api.feature_push(Gd, kind, P, R, 1e-5, alpha=0.1, beta=0.5 if kind == L.IGN else 0.0,
                               prec="fp64", tile_w=W)
        out.append((res["oper"], P.cpu().numpy(), R.cpu().numpy()))
    np.testing.assert_allclose(out[0][0], out[1][0], rtol=1e-12)
    np.testing.assert_allclose(out[0][1], out[1][1], rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(out[0][2], out[1][2], rtol=1e-10, atol=1e-14)
