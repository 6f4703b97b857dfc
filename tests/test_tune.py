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
    fast = tune.autotune(Gd, L.PPR, seeds, eps, shapes=shapes, buckets=[{}], use_cache=False, reps=1)
    assert fast["ms"] == min(t[1] for t in fast["table"])
    bound = min(t[2] for t in fast["table"]) * 1.05  # only the lowest-latency shapes qualify
    lat = tune.autotune(Gd, L.PPR, seeds, eps, shapes=shapes, buckets=[{}], use_cache=False, reps=1,
                        max_p99_ms=bound)
    ok = [t for t in lat["table"] if t[2] <= bound]
    assert ok and lat["p99_ms"] <= bound
    assert lat["ms"] == min(t[1] for t in ok)
