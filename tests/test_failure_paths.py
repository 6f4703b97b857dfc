"""Failure detection without a GPU fault: bounded device waits and the round cap.

Every device-side wait of the library is bounded.  The push kernel's grid
barrier and the edit dataflow's predecessor waits give up after a number of
polls, record GDE_EHANG and return, so the kernel ends and the context stays
usable.  These tests make the waits run out with a limit of a single poll
(``gde_ctx_set_wait_limit``), check the status, and check that the next call
with the default limit gives the oracle's results.  Nothing here faults,
traps or hangs the GPU: a waiter that gives up returns.

The round cap is the other failure path the reference never reaches (its
loops run until the stopping rule holds): ``max_rounds`` stops a solve with
GDE_EITERCAP.
"""
import numpy as np
import pytest

from gde import _lib as L
from gde import api, graphs
from oracle import oracle as O

from test_device_edit import _padded

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cl():
    g = graphs.chung_lu(3000, 2.1, 8.0, 300.0, seed=3)
    return g, api.Graph(g.indptr, g.indices)


@pytest.fixture
def limit_reset():
    yield
    api.set_wait_limit(0)


def test_grid_barrier_wait_runs_out_then_the_context_recovers(cl, limit_reset):
    g, Gd = cl
    deg = g.degree.astype(np.float64)
    seeds = graphs.uniform_seeds(g, 4, seed=31)
    api.set_wait_limit(1)
    with pytest.raises(L.GDEError) as ei:
        api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, 1e-6, prec="fp64", alpha=0.15, tile_w=4)
    assert ei.value.status == L.GDE_EHANG
    api.set_wait_limit(0)
    # the same solve, and a tracked-frontier method (Chebyshev: its marks were
    # written by the launch that stopped), both give the oracle's results
    res = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, 1e-6, prec="fp64", alpha=0.15, tile_w=4)
    che = api.solve(Gd, L.PPR, L.LOCAL_CHEBY, seeds, 1e-6, prec="fp64", alpha=0.15, tile_w=4)
    for i, s in enumerate(seeds):
        xo, _, oo = O.ppr_gd(g.n, g.indptr, g.indices, deg, int(s), 0.15, 1e-6, True)
        assert res["oper"][i] == pytest.approx(oo, rel=1e-12)
        assert np.abs(res["x"][i] - xo).sum() < 1e-12
        xc, _, oc = O.cheby(g.n, g.indptr, g.indices, deg, int(s), 0.15, 1e-6, True, sync=True)
        assert che["oper"][i] == pytest.approx(oc, rel=1e-12)
        assert np.abs(che["x"][i] - xc).sum() < 1e-10


def test_served_queue_wait_runs_out(cl, limit_reset):
    g, Gd = cl
    seeds = graphs.uniform_seeds(g, 40, seed=32)
    api.set_wait_limit(1)
    with pytest.raises(L.GDEError) as ei:
        api.serve(Gd, L.PPR, seeds, 1e-6, prec="fp32", alpha=0.1, slots=8)
    assert ei.value.status == L.GDE_EHANG
    api.set_wait_limit(0)
    res = api.serve(Gd, L.PPR, seeds, 1e-6, prec="fp32", alpha=0.1, slots=8)
    assert (res["oper"] > 0).all()


def _hub_chain(g, hub, count, seed):
    """count edges on `hub`, each pair twice in a row (insert then delete): every edge waits on the previous."""
    rng = np.random.default_rng(seed)
    others = rng.choice(np.setdiff1d(np.arange(g.n), [hub]), size=count // 2, replace=False)
    pairs = np.repeat(np.stack([np.full(len(others), hub), others], 1), 2, axis=0)
    return pairs[:, 0].astype(np.int32), pairs[:, 1].astype(np.int32)


def test_edit_dataflow_wait_runs_out_and_restores_the_rows(limit_reset):
    import torch
    g = graphs.chung_lu(3000, 2.2, 6.0, 120.0, seed=24)
    hub = int(np.argmax(np.diff(g.indptr)))
    us, vs = _hub_chain(g, hub, 2000, seed=7)
    ip, ix, dg = _padded(g, 16)
    ix0, dg0 = ix.copy(), dg.copy()
    alpha, eps = 0.1, 1e-5
    seeds = graphs.uniform_seeds(g, 2, seed=3)
    F = len(seeds)
    Po, Ro = np.zeros((F, g.n)), np.zeros((F, g.n))
    for f, s in enumerate(seeds):
        Ro[f, s] = alpha
    ixo, dgo = ix.copy(), dg.copy()
    O.update_ppr(g.n, ip, ixo, dgo, alpha, eps, 1.0, Po, Ro, np.zeros(0, np.int32), np.zeros(0, np.int32), sync=True)
    Gd = api.Graph(ip, ix, row_len=dg, degree=dg.astype(np.float64))
    P = torch.from_numpy(np.ascontiguousarray(Po.T)).cuda()
    R = torch.from_numpy(np.ascontiguousarray(Ro.T)).cuda()
    P0, R0 = P.clone(), R.clone()
    api.set_wait_limit(1)
    with pytest.raises(L.GDEError) as ei:
        api.feature_update(Gd, L.UPPR, ix, dg, us, vs, False, P, R, None, eps, alpha=alpha, prec="fp64", tile_w=1)
    assert ei.value.status == L.GDE_EHANG
    # nothing was applied: the caller's arrays and matrices are unchanged
    np.testing.assert_array_equal(ix, ix0)
    np.testing.assert_array_equal(dg, dg0)
    assert torch.equal(P, P0) and torch.equal(R, R0)
    # the device rows were restored: the same batch with the default limit is the sequential pass
    api.set_wait_limit(0)
    oo = O.update_ppr(g.n, ip, ixo, dgo, alpha, eps, 1.0, Po, Ro, us, vs, sync=True)
    res = api.feature_update(Gd, L.UPPR, ix, dg, us, vs, False, P, R, None, eps, alpha=alpha, prec="fp64", tile_w=1)
    assert res["stats"]["edit_path"] == 2  # the device dataflow ran
    np.testing.assert_array_equal(ix, ixo)
    np.testing.assert_array_equal(dg, dgo)
    np.testing.assert_allclose(res["oper"], oo, rtol=1e-12)
    np.testing.assert_allclose(P.cpu().numpy().T, Po, rtol=1e-9, atol=1e-13)
    np.testing.assert_allclose(R.cpu().numpy().T, Ro, rtol=1e-9, atol=1e-13)


@pytest.mark.parametrize("tile_w", [1, 4])
def test_round_cap_returns_itercap(cl, tile_w):
    g, Gd = cl
    seeds = graphs.uniform_seeds(g, 3, seed=33)
    with pytest.raises(L.GDEError) as ei:
        api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, 1e-7, prec="fp64", alpha=0.1, tile_w=tile_w, max_rounds=2)
    assert ei.value.status == L.GDE_EITERCAP
    # the context is usable afterwards and the uncapped solve is the oracle's
    deg = g.degree.astype(np.float64)
    res = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, 1e-7, prec="fp64", alpha=0.1, tile_w=tile_w)
    for i, s in enumerate(seeds):
        _, _, oo = O.ppr_gd(g.n, g.indptr, g.indices, deg, int(s), 0.1, 1e-7, True)
        assert res["oper"][i] == pytest.approx(oo, rel=1e-12)
