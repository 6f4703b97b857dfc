"""The autotuner's pick rule: fastest configuration, or fastest within a p99 latency bound."""
import numpy as np
import pytest

from gde import _lib as L
from gde import api, graphs, tune

pytestmark = pytest.mark.gpu


def test_autotune_with_and_without_a_latency_bound():
    g = graphs.chung_lu(20000, 2.1, 8.0, 500.0, seed=8)
    Gd = api.Graph(g.indptr, g.indices)
    seeds = graphs.uniform_seeds(g, 128, seed=3)
    eps = np.exp(np.random.default_rng(1).uniform(np.log(1e-7), np.log(1e-5), 128))
    shapes = [{"tile_w": 1, "slots": 16}, {"tile_w": 1, "slots": 64}, {"tile_w": 8}]
    fast = tune.autotune(Gd, L.PPR, seeds, eps, shapes=shapes, buckets=[{}], slots_per_group=[], use_cache=False,
                         reps=1)
    table = fast["table"]
    assert len(table) == 3 and all(len(t) == 3 for t in table)
    assert fast["ms"] == min(t[1] for t in table)
    # the rule on the measured table: fastest among the configurations within the bound
    bound = sorted(t[2] for t in table)[1]
    ok = [t for t in table if t[2] <= bound]
    best = tune._pick(table, bound)
    assert best[2] <= bound and best[1] == min(t[1] for t in ok)
    # no configuration within the bound: the one with the lowest p99
    assert tune._pick(table, 0.0)[2] == min(t[2] for t in table)
    # a live run with a bound every configuration meets keeps a configuration within it
    loose = tune.autotune(Gd, L.PPR, seeds, eps, shapes=shapes, buckets=[{}], slots_per_group=[], use_cache=False,
                          reps=1, max_p99_ms=1e9)
    assert loose["p99_ms"] <= 1e9 and loose["max_p99_ms"] == 1e9
    # a served winner is timed again with its slots sharing block groups
    grouped = tune.autotune(Gd, L.PPR, seeds, eps, shapes=shapes[1:2], buckets=[{}], slots_per_group=[8],
                            use_cache=False, reps=1)
    assert [t[0].get("groups") for t in grouped["table"]] == [None, 8]
