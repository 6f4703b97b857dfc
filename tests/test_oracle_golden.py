"""Pin the C oracle against the reference's own outputs (golden fixtures).

The fixtures were produced by running the reference's unmodified CPU code
(``tests/golden/make_golden.py``).  Because the oracle restates each function
with the same floating-point operation order, FP64 outputs must agree to the
last bit or nearly so; operation counts and graph edits must agree exactly.
"""
import numpy as np
import pytest

import golden_cases as G
from oracle import oracle as O

GRAPHS = G.graphs()


def _g(name):
    g = GRAPHS[name]
    return g["indptr"], g["indices"], np.diff(g["indptr"]).astype(np.float64)


def _close(a, b):
    np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-16)


@pytest.mark.parametrize("c", G.cases("ppr_gd"), ids=lambda c: c["id"])
def test_ppr_gd(c):
    ip, ix, d = _g(c["graph"])
    p = c["p"]
    x, r, oper = O.ppr_gd(len(ip) - 1, ip, ix, d, p["s"], p["alpha"], p["eps"], bool(p["local"]))
    assert oper == int(c["o"]["oper"])
    _close(x, c["o"]["x"])
    _close(r, c["o"]["r"])


@pytest.mark.parametrize("c", G.cases("ppr_cheby"), ids=lambda c: c["id"])
def test_ppr_cheby(c):
    ip, ix, d = _g(c["graph"])
    p = c["p"]
    x, r, oper = O.cheby(len(ip) - 1, ip, ix, d, p["s"], p["alpha"], p["eps"], bool(p["local"]))
    assert oper == int(c["o"]["oper"])
    _close(x, c["o"]["x"])
    _close(r, c["o"]["r"])


@pytest.mark.parametrize("c", G.cases("ppr_sor") + G.cases("katz_sor"), ids=lambda c: c["id"])
def test_sor(c):
    ip, ix, d = _g(c["graph"])
    p = c["p"]
    x, r, oper = O.sor(len(ip) - 1, ip, ix, d, p["s"], p["alpha"], p["eps"], p["omega"], bool(p["local"]),
                       katz=c["kind"] == "katz_sor")
    assert oper == float(c["o"]["oper"])
    _close(x, c["o"]["x"])
    _close(r, c["o"]["r"])


@pytest.mark.parametrize("c", G.cases("katz_gd"), ids=lambda c: c["id"])
def test_katz_gd(c):
    ip, ix, d = _g(c["graph"])
    p = c["p"]
    x, r, oper = O.katz_gd(len(ip) - 1, ip, ix, d, p["s"], p["alpha"], p["eps"], bool(p["local"]))
    assert oper == int(c["o"]["oper"])
    _close(x, c["o"]["x"])
    _close(r, c["o"]["r"])


@pytest.mark.parametrize("c", G.cases("katz_cheby"), ids=lambda c: c["id"])
def test_katz_cheby(c):
    ip, ix, d = _g(c["graph"])
    p = c["p"]
    x, r, oper = O.cheby(len(ip) - 1, ip, ix, d, p["s"], p["alpha"], p["eps"], bool(p["local"]), katz=True,
                         l_max=p["l_max"], mu_min=p["mu_min"])
    assert oper == int(c["o"]["oper"])
    _close(x, c["o"]["x"])
    _close(r, c["o"]["r"])


@pytest.mark.parametrize("c", G.cases("estimate_n"), ids=lambda c: c["id"])
def test_estimate_n(c):
    assert O.hk_estimate_n(c["p"]["tau"], c["p"]["eps"]) == int(c["o"]["n"])


@pytest.mark.parametrize("c", G.cases("hk_sor_queue"), ids=lambda c: c["id"])
def test_hk_sor_queue(c):
    ip, ix, d = _g(c["graph"])
    p = c["p"]
    est, x, r, oper = O.hk_sor_queue(len(ip) - 1, ip, ix, d, p["s"], p["tau"], p["eps"], p["omega"], bool(p["local"]))
    assert est == int(c["o"]["est_n"])
    assert oper == float(c["o"]["oper"])
    _close(x, c["o"]["x"])
    _close(r, c["o"]["r"])


@pytest.mark.parametrize("c", G.cases("hk_sor_queue"), ids=lambda c: c["id"])
def test_hk_sync_form_is_the_reference_where_order_cannot_matter(c):
    """The level-synchronous HK form (the GPU's) equals the reference's queue for omega = 1
    and for the global sweeps at any omega; only the local form with omega != 1 differs
    (its re-enqueue test reads the next level's queue marks)."""
    ip, ix, d = _g(c["graph"])
    p = c["p"]
    n = len(ip) - 1
    for omega in ((p["omega"],) if p["omega"] == 1.0 else (0.8, p["omega"])):
        for local in ((True, False) if omega == 1.0 else (False,)):
            e1, x1, _, o1 = O.hk_sor_queue(n, ip, ix, d, p["s"], p["tau"], p["eps"], omega, local)
            e2, x2, _, o2 = O.hk_sor_queue(n, ip, ix, d, p["s"], p["tau"], p["eps"], omega, local, sync=True)
            assert e1 == e2 and o1 == o2
            np.testing.assert_allclose(x2, x1, rtol=1e-12, atol=1e-16)


@pytest.mark.parametrize("c", [c for c in G.cases("hk_sor_queue") if c["p"]["omega"] != 1.0 and c["p"]["local"]],
                         ids=lambda c: c["id"])
def test_hk_sync_local_relaxation_keeps_the_heat_kernel_mass(c):
    """Relaxing each node to its threshold keeps sum(x) near 1 (the heat kernel is
    column-stochastic) and x near expm; the reference's local queue with omega != 1 leaves
    part of each (1 - omega) r unpushed."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    ip, ix, d = _g(c["graph"])
    p = c["p"]
    n = len(ip) - 1
    _, x, _, _ = O.hk_sor_queue(n, ip, ix, d, p["s"], p["tau"], p["eps"], p["omega"], True, sync=True)
    A = sp.csr_matrix((np.ones(len(ix)), ix, ip), shape=(n, n))
    Lap = (A @ sp.diags(1.0 / np.asarray(d, np.float64))) - sp.identity(n)
    e = np.zeros(n)
    e[p["s"]] = 1.0
    truth = spla.expm_multiply(p["tau"] * Lap.tocsc(), e)
    assert abs(x.sum() - 1.0) < 1e-2
    assert np.abs(x - truth).sum() < 1e-2
    assert np.abs(c["o"]["x"] - truth).sum() >= np.abs(x - truth).sum() - 1e-12


@pytest.mark.parametrize("c", G.cases("hk_taylor_approx"), ids=lambda c: c["id"])
def test_hk_taylor(c):
    ip, ix, d = _g(c["graph"])
    p = c["p"]
    est, x = O.hk_taylor(len(ip) - 1, ip, ix, d, p["s"], p["tau"], p["eps"])
    assert est == int(c["o"]["est_n"])
    _close(x, c["o"]["x"])


def _instantgnn_run(algo):
    dy = G.dyn()
    n = len(dy["indptr"]) - 1
    indptr = dy["indptr"].copy()
    indices = dy["indices"].astype(np.int32).copy()
    degree = dy["degree"].astype(np.int64).copy()
    X = dy["X"]
    static = [c for c in G.cases("instantgnn_static") if str(c["p"]["algo"]) == algo][0]
    updates = [c for c in G.cases("instantgnn_update") if str(c["p"]["algo"]) == algo]
    p = static["p"]
    P = np.zeros_like(X)
    R = X.copy()
    O.ign_static(n, indptr, indices, degree, p["alpha"], p["eps"], P, R, p["beta"], omega=p["omega"],
                 sor=algo.startswith("sor"))
    yield "static", (P, R), static
    for c in sorted(updates, key=lambda c: int(c["p"]["snap"])):
        O.ign_update(n, indptr, indices, degree, p["alpha"], p["eps"], p["omega"], P, R, X, c["o"]["us"],
                     c["o"]["vs"], p["beta"], algo)
        yield "update", (P, R, indices, degree), c


@pytest.mark.parametrize("algo", ["fwdbatchinsert", "sorbatchinsert", "fwdbatch"])
def test_instantgnn(algo):
    for stage, vals, c in _instantgnn_run(algo):
        _close(vals[0], c["o"]["P"])
        _close(vals[1], c["o"]["R"])
        if stage == "update":
            np.testing.assert_array_equal(vals[2], c["o"]["indices"])
            np.testing.assert_array_equal(vals[3], c["o"]["degree"])


def test_update_ppr():
    dy = G.dyn()
    n = len(dy["indptr"]) - 1
    indptr = dy["indptr"].copy()
    indices = dy["indices"].astype(np.int32).copy()
    degree = dy["degree"].astype(np.int64).copy()
    seeds = G.load()["dynppr/seeds"]
    cs = sorted(G.cases("update_ppr"), key=lambda c: int(c["p"]["snap"]))
    P = np.zeros((len(seeds), n))
    R = np.zeros((len(seeds), n))
    for f, s in enumerate(seeds):
        R[f, s] = cs[0]["p"]["alpha"]
    for c in cs:
        p = c["p"]
        snap = int(p["snap"])
        opers = O.update_ppr(n, indptr, indices, degree, p["alpha"], p["eps"], p["omega"], P, R,
                             dy["Us"][snap], dy["Vs"][snap])
        np.testing.assert_array_equal(opers, c["o"]["opers"])
        _close(P, c["o"]["P"])
        _close(R, c["o"]["R"])
        np.testing.assert_array_equal(indices, c["o"]["indices"])
        np.testing.assert_array_equal(degree, c["o"]["degree"])
