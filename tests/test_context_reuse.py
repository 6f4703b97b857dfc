"""One context serving graphs of different sizes, one after another.

The frontier dedup marks of tile t live at ``mark + t * n`` and are compared
for equality with a per-round stamp, so a graph of another size maps tile t
onto marks that another tile wrote.  Every tile of a launch therefore starts
past the largest stamp any tile has used.  These tests alternate graph sizes,
tile widths and the served / batched engines on one context and hold every
solve to the oracle's exact operation counts: a stale mark that equalled a
current stamp would drop a node from a frontier and change the count.
"""
import numpy as np
import pytest

from gde import _lib as L
from gde import api, graphs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_alternating_graph_sizes_keep_exact_operation_counts():
    gs = [graphs.chung_lu(n, 2.2, 6.0, 80.0, seed=50 + i) for i, n in enumerate((1500, 4000, 2500))]
    Gs = [api.Graph(g.indptr, g.indices) for g in gs]
    rng = np.random.default_rng(9)
    for step in range(9):
        i = int(rng.integers(0, 3))
        g, Gd = gs[i], Gs[i]
        W = [1, 4, 8][step % 3]
        seeds = graphs.uniform_seeds(g, 10, seed=step)
        eps = 1e-6
        if W == 1 and step % 2:
            res = api.serve(Gd, L.PPR, seeds, eps, alpha=0.15, prec="fp64", slots=3)
        else:
            res = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, eps, prec="fp64", alpha=0.15, tile_w=W)
        deg = g.degree.astype(np.float64)
        for q, s in enumerate(seeds):
            xo, _, oo = O.ppr_gd(g.n, g.indptr, g.indices, deg, int(s), 0.15, eps, True)
            assert res["oper"][q] == pytest.approx(oo, rel=1e-12), (step, i, W, q)
            assert np.abs(res["x"][q] - xo).sum() <= 1e-10 * np.abs(xo).sum(), (step, i, W, q)
