"""Edge batches with deletions applied on the device (dataflow over the batch).

``updetaGraph`` (InstantGNN.py:137-180) walks the batch in order: an edge
whose endpoint is already in the row is deleted (swap with the row's last
entry) when both endpoints keep a neighbour, otherwise it is appended to both
rows.  The device pass keeps that sequential meaning exactly: each edge waits
until every earlier edge that shares an endpoint has been applied.  These
tests check, on padded graphs with slack, that the device pass ran
(``gde_stats.edit_path``) and that the edited arrays, the repaired residuals
and the push are the same as the oracle's sequential pass.  Every batch
runs on the device: a batch whose insertion finds a row full applies the
edges before it and reports ``GDE_ECAPACITY``; self-loops follow the
sequential pass literally, and a self-loop insertion that would make a
padding slot part of its row reports ``GDE_EINVAL`` after the edges before
it.
"""
import numpy as np
import pytest

from gde import _lib as L
from gde import api, graphs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EDIT_DEVICE_DATAFLOW = 2


def _padded(g, slack):
    n = g.n
    deg = np.diff(g.indptr).astype(np.int64)
    ip = np.zeros(n + 1, np.int64)
    np.cumsum(deg + slack, out=ip[1:])
    ix = np.full(ip[-1], n, np.int32)
    for u in range(n):
        ix[ip[u]:ip[u] + deg[u]] = g.indices[g.indptr[u]:g.indptr[u + 1]]
    return ip, ix, deg


def _mixed_batch(g, k_del, k_ins, k_rep, seed, hub=None, hub_times=0):
    """Deletions of present edges, insertions of new pairs, some pairs twice (toggles), shuffled."""
    rng = np.random.default_rng(seed)
    n = g.n
    src = np.repeat(np.arange(n), np.diff(g.indptr))
    pick = rng.choice(len(src), size=k_del, replace=False)
    dels = np.stack([src[pick], g.indices[pick]], 1)
    ins = rng.integers(0, n, size=(k_ins, 2))
    ins = ins[ins[:, 0] != ins[:, 1]]
    rep = np.concatenate([dels, ins])[rng.choice(len(dels) + len(ins), size=k_rep)]
    e = np.concatenate([dels, ins, rep])
    e = e[rng.permutation(len(e))]
    if hub is not None:
        # the hub's edges come last, each pair twice in a row (insert, then delete again): the
        # row never grows by more than one entry, but the batch touches it hub_times times
        others = rng.choice(np.setdiff1d(np.arange(n), [hub]), size=hub_times // 2, replace=False)
        pairs = np.repeat(np.stack([np.full(len(others), hub), others], 1), 2, axis=0)
        e = np.concatenate([e, pairs])
    return e[:, 0].astype(np.int32), e[:, 1].astype(np.int32)


def _run_uppr(g, slack, us, vs, seeds, alpha=0.1, eps=1e-5):
    import torch
    n = g.n
    ip, ix, dg = _padded(g, slack)
    ix_o, dg_o = ix.copy(), dg.copy()
    F = len(seeds)
    Po = np.zeros((F, n))
    Ro = np.zeros((F, n))
    for f, s in enumerate(seeds):
        Ro[f, s] = alpha
    O.update_ppr(n, ip, ix_o, dg_o, alpha, eps, 1.0, Po, Ro, np.zeros(0, np.int32), np.zeros(0, np.int32), sync=True)
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    P = torch.from_numpy(np.ascontiguousarray(Po.T)).cuda()
    R = torch.from_numpy(np.ascontiguousarray(Ro.T)).cuda()
    oo = O.update_ppr(n, ip, ix_o, dg_o, alpha, eps, 1.0, Po, Ro, us, vs, sync=True)
    res = api.feature_update(Gd, L.UPPR, ix, dg, us, vs, False, P, R, None, eps, alpha=alpha, prec="fp64",
                             tile_w=1)
    np.testing.assert_array_equal(ix, ix_o)
    np.testing.assert_array_equal(dg, dg_o)
    np.testing.assert_allclose(res["oper"], oo, rtol=1e-12)
    np.testing.assert_allclose(P.cpu().numpy().T, Po, rtol=1e-9, atol=1e-13)
    np.testing.assert_allclose(R.cpu().numpy().T, Ro, rtol=1e-9, atol=1e-13)
    return res, Gd, ix, dg


def test_mixed_batch_runs_on_device_and_matches_sequential_pass():
    g = graphs.chung_lu(3000, 2.2, 6.0, 120.0, seed=21)
    us, vs = _mixed_batch(g, 400, 400, 120, seed=5)
    deg0 = np.diff(g.indptr)
    res, Gd, ix, dg = _run_uppr(g, 64, us, vs, graphs.uniform_seeds(g, 2, seed=3))
    assert res["stats"]["edit_path"] == EDIT_DEVICE_DATAFLOW
    assert (dg < deg0).any() and (dg > deg0).any()  # the batch both deleted and inserted


def test_mixed_batch_then_push_on_the_edited_graph_matches_a_fresh_upload():
    """After the device edit, the device copy of the graph (rows, degrees, tables) is the edited one."""
    import torch
    g = graphs.chung_lu(3000, 2.2, 6.0, 120.0, seed=23)
    us, vs = _mixed_batch(g, 300, 300, 60, seed=8)
    res, Gd, ix, dg = _run_uppr(g, 48, us, vs, graphs.uniform_seeds(g, 1, seed=4))
    assert res["stats"]["edit_path"] == EDIT_DEVICE_DATAFLOW
    ip, _, _ = _padded(g, 48)
    fresh = api.Graph(ip, ix.copy(), row_len=dg.copy(), degree=dg.astype(np.float64))
    seeds = graphs.uniform_seeds(g, 4, seed=9)
    a = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, 1e-7, prec="fp64", alpha=0.15, tile_w=1)
    b = api.solve(fresh, L.PPR, L.LOCAL_GD, seeds, 1e-7, prec="fp64", alpha=0.15, tile_w=1)
    np.testing.assert_allclose(a["x"], b["x"], rtol=1e-12, atol=1e-16)
    X = np.random.default_rng(2).standard_normal((g.n, 3))
    out = []
    for G in (Gd, fresh):
        P = torch.zeros(X.shape, dtype=torch.float64, device="cuda")
        R = torch.from_numpy(X.copy()).cuda()
        r = api.feature_push(G, L.IGN, P, R, 1e-4, alpha=0.1, beta=0.5, prec="fp64")
        out.append((r["oper"], P.cpu().numpy()))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_allclose(out[0][1], out[1][1], rtol=1e-12, atol=1e-15)


def test_row_touched_more_often_than_its_slack_stays_on_the_device():
    """The slack test is exact (made when an insertion runs), not a bound from the batch."""
    g = graphs.chung_lu(3000, 2.2, 6.0, 120.0, seed=22)
    hub = int(np.argmax(np.diff(g.indptr)))
    us, vs = _mixed_batch(g, 100, 100, 20, seed=6, hub=hub, hub_times=12)
    res, _, _, _ = _run_uppr(g, 4, us, vs, graphs.uniform_seeds(g, 2, seed=3))
    assert res["stats"]["edit_path"] == EDIT_DEVICE_DATAFLOW


def test_batch_that_fills_a_row_applies_the_edges_before_it_and_errors():
    """A row without slack for an insertion: the device run stops, the touched rows go back to the
    caller's arrays, the edges before that one run again on the device, and the error is reported."""
    import torch
    g = graphs.chung_lu(3000, 2.2, 6.0, 120.0, seed=24)
    n = g.n
    slack = 2
    ip, ix, dg = _padded(g, slack)
    rng = np.random.default_rng(17)
    us, vs = _mixed_batch(g, 150, 150, 30, seed=9)
    low = int(np.argmin(np.diff(g.indptr)))
    new = rng.choice(np.setdiff1d(np.arange(n), np.concatenate([[low], g.indices[g.indptr[low]:g.indptr[low + 1]]])),
                     size=slack + 1, replace=False)
    cut = len(us) // 2
    us = np.concatenate([us[:cut], np.full(slack + 1, low, np.int32), us[cut:]]).astype(np.int32)
    vs = np.concatenate([vs[:cut], new.astype(np.int32), vs[cut:]]).astype(np.int32)
    # the expected partial edit: the oracle, edge by edge, up to the insertion that finds a row full
    ix_o, dg_o = ix.copy(), dg.copy()
    stop = None
    for e in range(len(us)):
        u, v = int(us[e]), int(vs[e])
        row = ix_o[ip[u]:ip[u] + dg_o[u]]
        present = (row == v).any()
        if not present and (dg_o[u] >= ip[u + 1] - ip[u] or dg_o[v] >= ip[v + 1] - ip[v]):
            stop = e
            break
        O.update_graph(n, ip, ix_o, dg_o, us[e:e + 1], vs[e:e + 1], False)
    assert stop is not None and stop <= cut + slack
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    P = torch.zeros((n, 1), dtype=torch.float64, device="cuda")
    R = torch.zeros((n, 1), dtype=torch.float64, device="cuda")
    with pytest.raises(L.GDEError) as ei:
        api.feature_update(Gd, L.UPPR, ix, dg, us, vs, False, P, R, None, 1e-5, alpha=0.1, prec="fp64", tile_w=1)
    assert ei.value.status == L.GDE_ECAPACITY
    np.testing.assert_array_equal(ix, ix_o)
    np.testing.assert_array_equal(dg, dg_o)
    # the device copy holds the same partial edit
    fresh = api.Graph(ip, ix.copy(), row_len=dg.copy(), degree=dg.astype(np.float64))
    seeds = graphs.uniform_seeds(g, 3, seed=5)
    a = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, 1e-7, prec="fp64", alpha=0.15, tile_w=1)
    b = api.solve(fresh, L.PPR, L.LOCAL_GD, seeds, 1e-7, prec="fp64", alpha=0.15, tile_w=1)
    np.testing.assert_allclose(a["x"], b["x"], rtol=1e-12, atol=1e-16)


@pytest.mark.parametrize("algo", ["fwdbatch"])
def test_instantgnn_mixed_batch_on_device(algo):
    import torch
    g = graphs.chung_lu(2500, 2.2, 6.0, 100.0, seed=31)
    n = g.n
    us, vs = _mixed_batch(g, 250, 250, 50, seed=12)
    ip, ix, dg = _padded(g, 64)
    ix_o, dg_o = ix.copy(), dg.copy()
    X = np.random.default_rng(7).standard_normal((n, 2))
    alpha, eps, beta = 0.1, 1e-4, 0.5
    Po = np.zeros_like(X)
    Ro = X.copy()
    O.ign_sync(n, ip, ix_o, dg_o, alpha, eps, beta, Po, Ro)
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    P = torch.zeros(X.shape, dtype=torch.float64, device="cuda")
    R = torch.from_numpy(X.copy()).cuda()
    Xd = torch.from_numpy(X.copy()).cuda()
    api.feature_push(Gd, L.IGN, P, R, eps, alpha=alpha, beta=beta, prec="fp64")
    _, oo = O.ign_update(n, ip, ix_o, dg_o, alpha, eps, 1.0, Po, Ro, X, us, vs, beta, algo, sync=True)
    res = api.feature_update(Gd, L.IGN, ix, dg, us, vs, False, P, R, Xd, eps, alpha=alpha, beta=beta, prec="fp64")
    assert res["stats"]["edit_path"] == EDIT_DEVICE_DATAFLOW
    np.testing.assert_array_equal(ix, ix_o)
    np.testing.assert_array_equal(dg, dg_o)
    np.testing.assert_allclose(res["oper"], oo, rtol=1e-12)
    np.testing.assert_allclose(P.cpu().numpy(), Po, rtol=1e-9, atol=1e-13)
    np.testing.assert_allclose(R.cpu().numpy(), Ro, rtol=1e-9, atol=1e-13)


def _repad_numpy(ip, ix, dg, min_slack):
    """The expected relayout: each row's live entries first, capacity max(old, degree + slack)."""
    n = len(dg)
    cap = np.maximum(np.diff(ip), dg + min_slack)
    ip2 = np.zeros(n + 1, np.int64)
    np.cumsum(cap, out=ip2[1:])
    ix2 = np.full(ip2[-1], n, np.int32)
    for u in range(n):
        ix2[ip2[u]:ip2[u] + dg[u]] = ix[ip[u]:ip[u] + dg[u]]
    return ip2, ix2


def test_repad_grows_the_slack_of_full_rows_and_the_batch_then_runs_on_the_device():
    """A batch that needs more slack than a row has: GDE_ECAPACITY on the tight layout;
    after gde_graph_repad the same batch runs on the device and matches the oracle."""
    import torch
    g = graphs.chung_lu(2000, 2.2, 6.0, 100.0, seed=41)
    n = g.n
    ip, ix, dg = _padded(g, 0)
    low = int(np.argmin(np.diff(g.indptr)))
    rng = np.random.default_rng(3)
    others = rng.choice(np.setdiff1d(np.arange(n), np.concatenate([[low], g.indices[g.indptr[low]:g.indptr[low + 1]]])),
                        size=5, replace=False)
    us = np.full(5, low, np.int32)
    vs = others.astype(np.int32)
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    P = torch.zeros((n, 1), dtype=torch.float64, device="cuda")
    R = torch.zeros((n, 1), dtype=torch.float64, device="cuda")
    R[int(low), 0] = 0.1
    ix_before, dg_before = ix.copy(), dg.copy()
    with pytest.raises(L.GDEError) as ei:
        api.feature_update(Gd, L.UPPR, ix, dg, us, vs, False, P, R, None, 1e-5, alpha=0.1, prec="fp64", tile_w=1)
    assert ei.value.status == L.GDE_ECAPACITY
    # no slack anywhere: the first insertion already failed, nothing changed
    np.testing.assert_array_equal(ix, ix_before)
    np.testing.assert_array_equal(dg, dg_before)
    ip2, ix2 = api.repad(Gd, 8)
    eip, eix = _repad_numpy(ip, ix, dg, 8)
    np.testing.assert_array_equal(ip2, eip)
    np.testing.assert_array_equal(ix2, eix)
    # the same batch now runs on the device and matches the oracle's sequential pass
    ix_o, dg_o = ix2.copy(), dg.copy()
    Po = np.zeros((1, n))
    Ro = np.ascontiguousarray(R.cpu().numpy().T)
    oo = O.update_ppr(n, ip2, ix_o, dg_o, 0.1, 1e-5, 1.0, Po, Ro, us, vs, sync=True)
    res = api.feature_update(Gd, L.UPPR, ix2, dg, us, vs, False, P, R, None, 1e-5, alpha=0.1, prec="fp64", tile_w=1)
    assert res["stats"]["edit_path"] == EDIT_DEVICE_DATAFLOW
    np.testing.assert_array_equal(ix2, ix_o)
    np.testing.assert_array_equal(dg, dg_o)
    np.testing.assert_allclose(res["oper"], oo, rtol=1e-12)
    np.testing.assert_allclose(P.cpu().numpy().T, Po, rtol=1e-9, atol=1e-13)
    np.testing.assert_allclose(R.cpu().numpy().T, Ro, rtol=1e-9, atol=1e-13)


def test_repad_keeps_every_solve_the_same():
    g = graphs.chung_lu(2000, 2.2, 6.0, 100.0, seed=42)
    ip, ix, dg = _padded(g, 1)
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    seeds = graphs.uniform_seeds(g, 4, seed=1)
    a = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, 1e-7, prec="fp64", alpha=0.15, tile_w=1)
    ip2, ix2 = api.repad(Gd, 3)
    assert ip2[-1] == ip[-1] + 2 * g.n
    b = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, 1e-7, prec="fp64", alpha=0.15, tile_w=1)
    np.testing.assert_array_equal(a["oper"], b["oper"])
    np.testing.assert_allclose(a["x"], b["x"], rtol=1e-12, atol=1e-16)
    with pytest.raises(L.GDEError) as ei:
        api.repad(api.Graph(g.indptr, g.indices), 2)  # a static (relabelled) graph has no padded layout
    assert ei.value.status == L.GDE_EINVAL


def _tiny_padded(n, edges, slack):
    a = np.array([e[0] for e in edges] + [e[1] for e in edges], np.int64)
    b = np.array([e[1] for e in edges] + [e[0] for e in edges], np.int64)
    order = np.lexsort((b, a))
    a, b = a[order], b[order]
    deg = np.bincount(a, minlength=n).astype(np.int64)
    ip = np.zeros(n + 1, np.int64)
    np.cumsum(deg + slack, out=ip[1:])
    ix = np.full(ip[-1], n, np.int32)
    fill = ip[:-1].copy()
    for x, y in zip(a, b):
        ix[fill[x]] = y
        fill[x] += 1
    return ip, ix, deg


@pytest.mark.parametrize("case", ["leaf_guard", "toggle", "swap_with_last", "star_hub"])
def test_device_edit_rules_on_tiny_graphs(case):
    """updetaGraph's rules one by one (InstantGNN.py:147-179), on the device path: the degree-1
    guard keeps an edge, a pair toggles delete / insert / delete, a deletion moves the row's last
    entry into the hole, and a hub's row takes a long chain of edits in batch order."""
    import torch
    if case == "leaf_guard":       # path 0-1-2-3: (0,1) has a leaf end, (1,2) does not
        n, edges, us, vs = 4, [(0, 1), (1, 2), (2, 3)], [0, 1, 2], [1, 2, 1]
    elif case == "toggle":
        n, edges, us, vs = 5, [(0, 1), (1, 2), (2, 3), (3, 4), (4, 0)], [0, 0, 2, 0, 2], [2, 2, 0, 2, 4]
    elif case == "swap_with_last":
        n, edges, us, vs = 6, [(0, 1), (0, 2), (0, 3), (0, 4), (1, 2), (2, 3), (3, 4), (4, 5), (5, 1)], \
            [0, 0, 3, 0], [1, 3, 2, 5]
    else:                          # star: centre 0 with 12 leaves, plus a ring on the leaves
        n = 13
        edges = [(0, i) for i in range(1, 13)] + [(i, i % 12 + 1) for i in range(1, 13)]
        rng = np.random.default_rng(5)
        pairs = [(0, int(v)) for v in rng.integers(1, 13, size=40)]
        us = [p[0] if i % 2 else p[1] for i, p in enumerate(pairs)]
        vs = [p[1] if i % 2 else p[0] for i, p in enumerate(pairs)]
    ip, ix, dg = _tiny_padded(n, edges, 6)
    us = np.asarray(us, np.int32)
    vs = np.asarray(vs, np.int32)
    ix_o, dg_o = ix.copy(), dg.copy()
    O.update_graph(n, ip, ix_o, dg_o, us, vs, False)
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    P = torch.zeros((n, 1), dtype=torch.float64, device="cuda")
    R = torch.zeros((n, 1), dtype=torch.float64, device="cuda")
    res = api.feature_update(Gd, L.UPPR, ix, dg, us, vs, False, P, R, None, 1e-3, alpha=0.2, prec="fp64", tile_w=1)
    assert res["stats"]["edit_path"] == EDIT_DEVICE_DATAFLOW
    np.testing.assert_array_equal(ix, ix_o)
    np.testing.assert_array_equal(dg, dg_o)


def _loop_graph(slack=4):
    """A 12-node ring with three chords, padded; node 3 carries a self-loop entry the way the
    reference's data format stores one (one slot, one degree, data_process_GNN.py:103-105)."""
    n = 12
    edges = [(i, (i + 1) % n) for i in range(n)] + [(0, 6), (2, 8), (4, 10)]
    ip, ix, dg = _tiny_padded(n, edges, slack)
    ix[ip[3] + dg[3]] = 3
    dg[3] += 1
    return n, ip, ix, dg


def _edit_and_push(n, ip, ix, dg, us, vs, only_insert, Gd=None):
    """gde_feature_update (PPR update, FP64) against the oracle's sequential edit + synchronous push."""
    import torch
    us = np.asarray(us, np.int32)
    vs = np.asarray(vs, np.int32)
    ix_o, dg_o = ix.copy(), dg.copy()
    F = 2
    Po = np.zeros((F, n))
    Ro = np.zeros((F, n))
    Ro[0, 1] = 0.2
    Ro[1, 7] = 0.2
    if Gd is None:
        Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    P = torch.from_numpy(np.ascontiguousarray(Po.T)).cuda()
    R = torch.from_numpy(np.ascontiguousarray(Ro.T)).cuda()
    oo = O.update_ppr(n, ip, ix_o, dg_o, 0.2, 1e-4, 1.0, Po, Ro, us, vs, sync=True)
    res = api.feature_update(Gd, L.UPPR, ix, dg, us, vs, only_insert, P, R, None, 1e-4, alpha=0.2, prec="fp64",
                             tile_w=1)
    assert res["stats"]["edit_path"] == EDIT_DEVICE_DATAFLOW
    np.testing.assert_array_equal(ix, ix_o)
    np.testing.assert_array_equal(dg, dg_o)
    np.testing.assert_allclose(res["oper"], oo, rtol=1e-12)
    np.testing.assert_allclose(P.cpu().numpy().T, Po, rtol=1e-9, atol=1e-13)
    np.testing.assert_allclose(R.cpu().numpy().T, Ro, rtol=1e-9, atol=1e-13)
    return Gd


def test_self_loop_deletion_on_the_device():
    """(3, 3) on a row that holds its loop: the loop leaves, every other 3 in the row takes the
    row's last entry, and the degree drops by two (InstantGNN.py:159-164)."""
    n, ip, ix, dg = _loop_graph()
    _edit_and_push(n, ip, ix, dg, [1, 3, 5], [7, 3, 9], False)


def test_self_loop_insertion_over_a_stale_slot_matches_the_sequential_pass():
    """Two deletions leave node 0's old entries behind its row; (0, 0) then writes one slot and
    counts two degrees, so the second slot's stale id joins the row, as in the reference."""
    n, ip, ix, dg = _loop_graph()
    Gd = _edit_and_push(n, ip, ix, dg, [0, 0], [1, 11], False)
    assert dg[0] == 1
    _edit_and_push(n, ip, ix, dg, [0, 2], [0, 9], False, Gd)
    assert dg[0] == 3 and ix[ip[0] + 1] == 0 and ix[ip[0] + 2] < n


def test_insert_only_batch_with_self_loops_on_the_device():
    """An insert-only batch with self-loops runs as the dataflow: (3, 3) on the loop's row is
    kept; the stale-slot insertion of a self-loop matches the sequential pass."""
    n, ip, ix, dg = _loop_graph()
    Gd = _edit_and_push(n, ip, ix, dg, [0, 0], [1, 11], False)
    us = np.array([3, 5, 0], np.int32)
    vs = np.array([3, 1, 0], np.int32)
    ix_o, dg_o = ix.copy(), dg.copy()
    O.update_graph(n, ip, ix_o, dg_o, us, vs, True)
    res = api.graph_update(Gd, ix, dg, us, vs, True)
    assert res["stats"]["edit_path"] == EDIT_DEVICE_DATAFLOW
    np.testing.assert_array_equal(res["outcome"], [0, 1, 1])
    np.testing.assert_array_equal(ix, ix_o)
    np.testing.assert_array_equal(dg, dg_o)
    fresh = api.Graph(ip, ix.copy(), row_len=dg.copy(), degree=dg.astype(np.float64))
    a = api.solve(Gd, L.PPR, L.LOCAL_GD, [0, 5], 1e-6, prec="fp64", alpha=0.15, tile_w=1)
    b = api.solve(fresh, L.PPR, L.LOCAL_GD, [0, 5], 1e-6, prec="fp64", alpha=0.15, tile_w=1)
    np.testing.assert_array_equal(a["oper"], b["oper"])
    np.testing.assert_allclose(a["x"], b["x"], rtol=1e-12, atol=1e-16)


@pytest.mark.parametrize("only_insert", [False, True])
def test_self_loop_insertion_over_the_padding_sentinel_is_an_error(only_insert):
    """(7, 7) on a row whose next free slots hold the sentinel n: the reference would make the
    sentinel part of the row and its next push would read it as a node id.  The edges before it
    stay applied, the error is GDE_EINVAL, and the device graph equals a fresh upload."""
    import torch
    n, ip, ix, dg = _loop_graph()
    us = np.array([1, 7, 2], np.int32)
    vs = np.array([5, 7, 9], np.int32)
    ix_o, dg_o = ix.copy(), dg.copy()
    O.update_graph(n, ip, ix_o, dg_o, us[:1], vs[:1], only_insert)
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    P = torch.zeros((n, 1), dtype=torch.float64, device="cuda")
    R = torch.zeros((n, 1), dtype=torch.float64, device="cuda")
    with pytest.raises(L.GDEError) as ei:
        api.feature_update(Gd, L.UPPR, ix, dg, us, vs, only_insert, P, R, None, 1e-4, alpha=0.2, prec="fp64",
                           tile_w=1)
    assert ei.value.status == L.GDE_EINVAL
    np.testing.assert_array_equal(ix, ix_o)
    np.testing.assert_array_equal(dg, dg_o)
    fresh = api.Graph(ip, ix.copy(), row_len=dg.copy(), degree=dg.astype(np.float64))
    a = api.solve(Gd, L.PPR, L.LOCAL_GD, [1, 7], 1e-6, prec="fp64", alpha=0.15, tile_w=1)
    b = api.solve(fresh, L.PPR, L.LOCAL_GD, [1, 7], 1e-6, prec="fp64", alpha=0.15, tile_w=1)
    np.testing.assert_array_equal(a["oper"], b["oper"])
    np.testing.assert_allclose(a["x"], b["x"], rtol=1e-12, atol=1e-16)


def test_endpoint_out_of_range_edits_nothing():
    import torch
    n, ip, ix, dg = _loop_graph()
    ix0, dg0 = ix.copy(), dg.copy()
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    P = torch.zeros((n, 1), dtype=torch.float64, device="cuda")
    R = torch.zeros((n, 1), dtype=torch.float64, device="cuda")
    for bad in (n, -1):
        with pytest.raises(L.GDEError) as ei:
            api.feature_update(Gd, L.UPPR, ix, dg, np.array([1, bad], np.int32), np.array([5, 2], np.int32), False,
                               P, R, None, 1e-4, alpha=0.2, prec="fp64", tile_w=1)
        assert ei.value.status == L.GDE_EINVAL
        np.testing.assert_array_equal(ix, ix0)
        np.testing.assert_array_equal(dg, dg0)


def test_insert_only_batch_that_fills_a_row_applies_the_edges_before_it():
    """An insert-only batch whose parallel pass finds a row full runs as the dataflow, which
    applies the edges before the failing insertion and reports GDE_ECAPACITY."""
    import torch
    n, ip, ix, dg = _loop_graph(slack=2)
    us = np.array([1, 2, 1, 1, 4], np.int32)
    vs = np.array([5, 6, 7, 9, 8], np.int32)  # node 1 takes a third insertion with two free slots
    ix_o, dg_o = ix.copy(), dg.copy()
    O.update_graph(n, ip, ix_o, dg_o, us[:3], vs[:3], True)
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    P = torch.zeros((n, 1), dtype=torch.float64, device="cuda")
    R = torch.zeros((n, 1), dtype=torch.float64, device="cuda")
    with pytest.raises(L.GDEError) as ei:
        api.feature_update(Gd, L.UPPR, ix, dg, us, vs, True, P, R, None, 1e-4, alpha=0.2, prec="fp64", tile_w=1)
    assert ei.value.status == L.GDE_ECAPACITY
    np.testing.assert_array_equal(ix, ix_o)
    np.testing.assert_array_equal(dg, dg_o)


def test_upload_rejects_the_padding_sentinel_inside_a_row():
    n, ip, ix, dg = _loop_graph()
    ix[ip[4] + 1] = n
    with pytest.raises(L.GDEError) as ei:
        api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    assert ei.value.status == L.GDE_EINVAL
