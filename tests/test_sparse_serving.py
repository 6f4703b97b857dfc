"""Served small queries out of hash tables (gde_params.sparse_blocks).

Queries with eps >= sparse_eps are solved by blocks that keep the touched
nodes in an open-addressing table with FP64 residuals and solutions, while
the other blocks run the dense FP32 slots.  The table path runs the same
synchronous rounds as the reference's local GD (ppr_solver.py:246-288,
katz_solver.py:206-243) in FP64, so its operation counts equal the FP64
oracle's exactly and its solutions match to FP32 output rounding.  A query
whose touched set outgrows 3/4 of its table is handed to the dense slots.
"""
import numpy as np
import pytest

from gde import _lib as L
from gde import api, graphs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# FP32 rows of FP64 values: relative rounding 2^-24 per entry
TABLE_L1 = 1e-6
# dense FP32 slots: rounding plus threshold flips at the largest degree
DENSE_MEAN_L1 = 2e-6


@pytest.fixture(scope="module")
def cl():
    g = graphs.chung_lu(3000, 2.1, 8.0, 300.0, seed=3)
    return g, api.Graph(g.indptr, g.indices)


def rel_l1(a, b):
    return np.abs(np.asarray(a, np.float64) - b).sum() / max(np.abs(b).sum(), 1e-300)


def oracle_row(g, kind, s, alpha, eps):
    deg = g.degree.astype(np.float64)
    fn = O.ppr_gd if kind == L.PPR else O.katz_gd
    x, _, oper = fn(g.n, g.indptr, g.indices, deg, int(s), alpha, eps, True)  # Katz x has x[s] -= 1 applied
    return x, oper


def alpha_of(g, kind):
    return 0.1 if kind == L.PPR else 1.0 / (float(g.degree.max()) + 1.0)


@pytest.mark.parametrize("kind", [L.PPR, L.KATZ])
def test_table_queries_match_the_fp64_oracle(cl, kind):
    g, Gd = cl
    alpha = alpha_of(g, kind)
    rng = np.random.default_rng(31)
    nq = 40
    seeds = graphs.uniform_seeds(g, nq, seed=31)
    eps = np.exp(rng.uniform(np.log(1e-7), np.log(1e-4), nq))
    cut = 1e-5
    res = api.serve(Gd, kind, seeds, eps, prec="fp32", alpha=alpha, slots=4,
                    tuning={"sparse_blocks": 6, "sparse_eps": cut})
    small = eps >= cut
    assert res["stats"]["sparse_queries"] == int(small.sum())
    assert res["stats"]["sparse_overflows"] == 0
    dense_errs = []
    for i, s in enumerate(seeds):
        xo, oo = oracle_row(g, kind, s, alpha, eps[i])
        err = rel_l1(res["x"][i], xo)
        if small[i]:
            assert res["oper"][i] == oo, (i, res["oper"][i], oo)
            assert err < TABLE_L1, (i, err)
        else:
            dense_errs.append(err)
    assert np.mean(dense_errs) < DENSE_MEAN_L1, dense_errs


def test_table_query_same_alone_and_in_the_mix(cl):
    g, Gd = cl
    rng = np.random.default_rng(32)
    nq = 24
    seeds = graphs.uniform_seeds(g, nq, seed=32)
    eps = np.exp(rng.uniform(np.log(1e-6), np.log(1e-4), nq))
    arrival = np.cumsum(rng.exponential(0.02, nq))
    tun = {"sparse_blocks": 3, "sparse_eps": 1e-5}
    mixed = api.serve(Gd, L.PPR, seeds, eps, arrival_ms=arrival, prec="fp32", alpha=0.1, slots=3, tuning=tun)
    assert (mixed["latency_ms"] > 0).all()
    for i in np.flatnonzero(eps >= 1e-5):
        alone = api.serve(Gd, L.PPR, seeds[i:i + 1], eps[i:i + 1], prec="fp32", alpha=0.1, slots=1, tuning=tun)
        assert alone["stats"]["sparse_queries"] == 1
        assert mixed["oper"][i] == alone["oper"][0], i
        assert mixed["rounds"][i] == alone["rounds"][0], i
        assert rel_l1(mixed["x"][i], alone["x"][0].astype(np.float64)) < TABLE_L1, i


def test_overflowing_queries_finish_in_dense_slots(cl):
    """A 1,024-entry table holds 768 nodes: larger touched sets move to the dense slots."""
    g, Gd = cl
    nq = 20
    seeds = graphs.uniform_seeds(g, nq, seed=33)
    eps = np.full(nq, 1e-6)
    res = api.serve(Gd, L.PPR, seeds, eps, prec="fp32", alpha=0.1, slots=3,
                    tuning={"sparse_blocks": 4, "sparse_eps": 1e-7, "sparse_cap": 1024})
    st = res["stats"]
    assert st["sparse_overflows"] > 0
    assert st["sparse_queries"] + st["sparse_overflows"] == nq
    errs = []
    for i, s in enumerate(seeds):
        xo, oo = oracle_row(g, L.PPR, s, 0.1, eps[i])
        err = rel_l1(res["x"][i], xo)
        # every query is complete whichever path finished it
        assert err < DENSE_MEAN_L1 + 6e-7 * float(g.degree.max()), (i, err)
        assert abs(res["oper"][i] - oo) <= 1e-3 * oo, (i, res["oper"][i], oo)
        errs.append(err)
    assert np.mean(errs) < DENSE_MEAN_L1, errs


def test_mixed_kinds_with_tables(cl):
    """Heat-kernel queries stay in the dense slots; small PPR / Katz ones go to tables."""
    g, Gd = cl
    rng = np.random.default_rng(34)
    nq = 18
    kinds = np.array([L.PPR, L.KATZ, L.HK] * (nq // 3), dtype=np.int32)
    rng.shuffle(kinds)
    seeds = graphs.uniform_seeds(g, nq, seed=34)
    eps = np.exp(rng.uniform(np.log(1e-6), np.log(1e-4), nq))
    katz_alpha = alpha_of(g, L.KATZ)
    alphas = np.where(kinds == L.KATZ, katz_alpha, 0.1)
    tau = 5.0
    res = api.serve_mixed(Gd, kinds, seeds, eps, alphas=alphas, tau=tau, prec="fp32", slots=4,
                          tuning={"sparse_blocks": 4, "sparse_eps": 1e-5})
    table = (kinds != L.HK) & (eps >= 1e-5)
    assert res["stats"]["sparse_queries"] == int(table.sum())
    for i in range(nq):
        if kinds[i] == L.HK:
            alone = api.solve(Gd, L.HK, L.HK_LOCAL, seeds[i:i + 1], eps[i:i + 1], prec="fp64", tau=tau, want_r=False)
            assert rel_l1(res["x"][i], alone["x"][0]) < 1e-4, i
            continue
        xo, oo = oracle_row(g, int(kinds[i]), seeds[i], float(alphas[i]), eps[i])
        if table[i]:
            assert res["oper"][i] == oo, i
            assert rel_l1(res["x"][i], xo) < TABLE_L1, i
        else:
            assert rel_l1(res["x"][i], xo) < 1e-4, i


def test_round_cap_reaches_the_caller_from_a_table_query(cl):
    """A table query that hits max_rounds moves to a dense slot, which reports the cap."""
    g, Gd = cl
    seeds = graphs.uniform_seeds(g, 4, seed=35)
    with pytest.raises(L.GDEError) as ei:
        api.serve(Gd, L.PPR, seeds, 1e-5, prec="fp32", alpha=0.1, slots=2, max_rounds=2,
                  tuning={"sparse_blocks": 2, "sparse_eps": 1e-6})
    assert ei.value.status == L.GDE_EITERCAP


def test_tables_off_without_solution_slabs(cl):
    """Residual rows need the dense slots: with want_r the switch is ignored."""
    g, Gd = cl
    seeds = graphs.uniform_seeds(g, 6, seed=36)
    res = api.serve(Gd, L.PPR, seeds, 1e-5, prec="fp32", alpha=0.1, want_r=True, slots=2,
                    tuning={"sparse_blocks": 2, "sparse_eps": 1e-6})
    assert res["stats"]["sparse_queries"] == 0
    deg = g.degree.astype(np.float64)
    for i in range(len(seeds)):
        assert (np.abs(res["r"][i].astype(np.float64)) < 1e-5 * 0.1 * deg * (1 + 1e-5)).all(), i
