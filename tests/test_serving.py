"""Continuous batching: a served query's result is the same alone and in the mix.

Queries with different seeds and eps arrive over time (Poisson gaps) into
fewer slots than queries, so later queries are admitted while earlier ones
are still pushing, and their work overlaps on the device.  Each result must
match the same query solved alone: FP64 exactly in operation count and to
1e-12 in x, FP32 within the flip-aware FP32 bound against the FP64 oracle.
"""
import numpy as np
import pytest

from gde import _lib as L
from gde import api, graphs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_L1 = 1e-12
FP32_MEAN_L1 = 2e-6


@pytest.fixture(scope="module")
def cl():
    g = graphs.chung_lu(3000, 2.1, 8.0, 300.0, seed=3)
    return g, api.Graph(g.indptr, g.indices)


def rel_l1(a, b):
    return np.abs(np.asarray(a, np.float64) - b).sum() / max(np.abs(b).sum(), 1e-300)


def mix(g, nq, seed):
    rng = np.random.default_rng(seed)
    seeds = graphs.uniform_seeds(g, nq, seed=seed)
    eps = np.exp(rng.uniform(np.log(1e-7), np.log(1e-5), nq))
    arrival = np.cumsum(rng.exponential(0.02, nq))  # ms
    return seeds, eps, arrival


@pytest.mark.parametrize("kind", [L.PPR, L.KATZ])
def test_served_fp64_same_alone_and_in_mix(cl, kind):
    g, Gd = cl
    alpha = 0.1 if kind == L.PPR else 1.0 / (float(g.degree.max()) + 1.0)
    seeds, eps, arrival = mix(g, 24, 5)
    served = api.serve(Gd, kind, seeds, eps, arrival_ms=arrival, prec="fp64", alpha=alpha, slots=4)
    assert (served["latency_ms"] > 0).all()
    for i in range(len(seeds)):
        alone = api.solve(Gd, kind, L.LOCAL_GD, seeds[i:i + 1], eps[i:i + 1], prec="fp64", alpha=alpha, tile_w=1)
        assert served["oper"][i] == pytest.approx(alone["oper"][0], rel=1e-12), i
        assert served["rounds"][i] == alone["rounds"][0], i
        assert rel_l1(served["x"][i], alone["x"][0]) < FP64_L1, i


def test_served_fp32_in_mix_matches_fp64_oracle(cl):
    g, Gd = cl
    deg = g.degree.astype(np.float64)
    seeds, eps, arrival = mix(g, 16, 9)
    served = api.serve(Gd, L.PPR, seeds, eps, arrival_ms=arrival, prec="fp32", alpha=0.1, slots=3)
    errs = []
    for i, s in enumerate(seeds):
        xo, _, oo = O.ppr_gd(g.n, g.indptr, g.indices, deg, int(s), 0.1, eps[i], True)
        err = rel_l1(served["x"][i], xo)
        # a few threshold flips at the largest degree (see test_gpu_parity)
        assert err < FP32_MEAN_L1 + 6 * eps[i] * 0.1 * float(g.degree.max()), (i, err)
        errs.append(err)
    assert np.mean(errs) < FP32_MEAN_L1, errs


def test_served_queries_wait_for_their_arrival(cl):
    g, Gd = cl
    seeds = graphs.uniform_seeds(g, 6, seed=2)
    arrival = np.array([0.0, 0.0, 5.0, 5.0, 10.0, 10.0])
    served = api.serve(Gd, L.PPR, seeds, 1e-6, arrival_ms=arrival, prec="fp32", alpha=0.1, slots=6)
    # the launch lasts at least until the last arrival; latency is counted from arrival
    assert served["stats"]["kernel_ms"] >= 10.0
    assert (served["latency_ms"] < 10.0).all()
