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


def test_served_mixed_kinds_same_alone(cl):
    """PPR, Katz and heat-kernel queries in one served launch, arriving over time."""
    g, Gd = cl
    rng = np.random.default_rng(4)
    nq = 18
    kinds = np.array([L.PPR, L.KATZ, L.HK] * (nq // 3), dtype=np.int32)
    rng.shuffle(kinds)
    seeds = graphs.uniform_seeds(g, nq, seed=21)
    eps = np.exp(rng.uniform(np.log(1e-6), np.log(1e-5), nq))
    katz_alpha = 1.0 / (float(g.degree.max()) + 1.0)
    alphas = np.where(kinds == L.KATZ, katz_alpha, 0.1)
    tau = 5.0
    arrival = np.cumsum(rng.exponential(0.03, nq))
    served = api.serve_mixed(Gd, kinds, seeds, eps, alphas=alphas, tau=tau, arrival_ms=arrival, prec="fp64", slots=5)
    for i in range(nq):
        if kinds[i] == L.HK:
            alone = api.solve(Gd, L.HK, L.HK_LOCAL, seeds[i:i + 1], eps[i:i + 1], prec="fp64", tau=tau, want_r=False)
        else:
            alone = api.solve(Gd, int(kinds[i]), L.LOCAL_GD, seeds[i:i + 1], eps[i:i + 1], prec="fp64",
                              alpha=float(alphas[i]), tile_w=1, want_r=False)
        assert served["oper"][i] == pytest.approx(alone["oper"][0], rel=1e-12), (i, int(kinds[i]))
        assert rel_l1(served["x"][i], alone["x"][0]) < 1e-11, (i, int(kinds[i]))


def test_served_mixed_hbm_budget_caps_slots(cl):
    g, Gd = cl
    seeds = graphs.uniform_seeds(g, 8, seed=4)
    kinds = np.full(8, L.PPR, dtype=np.int32)
    # about two slots' worth of vectors (FP32: ~45 B per node plus the chunk list)
    two = 2.5 * (45 * g.n + 16 * (g.nnz // 64 + 64))
    res = api.serve_mixed(Gd, kinds, seeds, 1e-6, alphas=0.1, hbm_budget_bytes=two, slots=8)
    assert res["stats"]["tiles"] == 2
    ref = api.serve(Gd, L.PPR, seeds, 1e-6, alpha=0.1, slots=8)
    np.testing.assert_allclose(res["oper"], ref["oper"], rtol=1e-3)
    with pytest.raises(L.GDEError) as ei:
        api.serve_mixed(Gd, kinds, seeds, 1e-6, alphas=0.1, hbm_budget_bytes=1000.0)
    assert ei.value.status == L.GDE_ENOMEM


def test_served_fp32_mixed_kinds_close_to_fp64(cl):
    """FP32 slots (interleaved {x, Kahan term} solution slabs kept per query and
    read out after the launch): PPR, Katz and heat kernel against FP64 alone."""
    g, Gd = cl
    rng = np.random.default_rng(6)
    nq = 15
    kinds = np.array([L.PPR, L.KATZ, L.HK] * (nq // 3), dtype=np.int32)
    rng.shuffle(kinds)
    seeds = graphs.uniform_seeds(g, nq, seed=23)
    eps = np.exp(rng.uniform(np.log(1e-6), np.log(1e-5), nq))
    katz_alpha = 1.0 / (float(g.degree.max()) + 1.0)
    alphas = np.where(kinds == L.KATZ, katz_alpha, 0.1)
    tau = 5.0
    served = api.serve_mixed(Gd, kinds, seeds, eps, alphas=alphas, tau=tau, prec="fp32", slots=4)
    for i in range(nq):
        if kinds[i] == L.HK:
            alone = api.solve(Gd, L.HK, L.HK_LOCAL, seeds[i:i + 1], eps[i:i + 1], prec="fp64", tau=tau, want_r=False)
        else:
            alone = api.solve(Gd, int(kinds[i]), L.LOCAL_GD, seeds[i:i + 1], eps[i:i + 1], prec="fp64",
                              alpha=float(alphas[i]), tile_w=1, want_r=False)
        # FP32 rounding plus a few threshold flips; a wrong row order, seed
        # correction or e^tau scale would be off by O(1)
        assert rel_l1(served["x"][i], alone["x"][0]) < 1e-4, (i, int(kinds[i]))


def test_served_fp32_residual_rows_meet_the_stopping_rule(cl):
    """Served FP32 residual rows come back in caller order: every entry is below
    its own eps * alpha * d_u, and x and r keep the PPR mass identity."""
    g, Gd = cl
    seeds = graphs.uniform_seeds(g, 10, seed=24)
    eps = 1e-6
    served = api.serve(Gd, L.PPR, seeds, eps, alpha=0.1, prec="fp32", want_r=True, slots=3)
    deg = g.degree.astype(np.float64)
    for i in range(len(seeds)):
        x = served["x"][i].astype(np.float64)
        r = served["r"][i].astype(np.float64)
        assert (np.abs(r) < eps * 0.1 * deg * (1 + 1e-5)).all(), i
        assert abs(x.sum() + r.sum() / 0.1 - 1.0) < 1e-5, i


def test_served_rows_into_pinned_host_memory(cl):
    """Pinned host rows are written directly by the device; pageable rows go through staging."""
    import torch
    g, Gd = cl
    seeds = graphs.uniform_seeds(g, 12, seed=25)
    pinned = torch.zeros((12, g.n), dtype=torch.float32).pin_memory()
    a = api.serve(Gd, L.PPR, seeds, 1e-6, alpha=0.1, prec="fp32", x_out=pinned, device_out=False, slots=4)
    b = api.serve(Gd, L.PPR, seeds, 1e-6, alpha=0.1, prec="fp32", slots=4)  # numpy rows
    np.testing.assert_allclose(a["oper"], b["oper"], rtol=1e-3)
    for i in range(12):
        assert rel_l1(pinned[i].numpy(), b["x"][i].astype(np.float64)) < 1e-5, i


@pytest.mark.parametrize("arrivals", [False, True])
@pytest.mark.parametrize("groups", [2, 4])
def test_slot_groups_give_the_same_results(cl, groups, arrivals):
    """Slots split over block groups with their own barriers: every query still equals the query alone."""
    g, Gd = cl
    seeds, eps, arrival = mix(g, 40, 11)
    served = api.serve(Gd, L.PPR, seeds, eps, arrival_ms=arrival if arrivals else None, prec="fp64", alpha=0.1,
                       slots=8, tuning={"groups": groups})
    one = api.serve(Gd, L.PPR, seeds, eps, prec="fp64", alpha=0.1, slots=8, tuning={"groups": 1})
    np.testing.assert_allclose(served["oper"], one["oper"], rtol=1e-12)
    np.testing.assert_array_equal(served["rounds"], one["rounds"])
    for i in range(len(seeds)):
        assert rel_l1(served["x"][i], one["x"][i]) < FP64_L1, i
    mixed = api.serve_mixed(Gd, [L.PPR, L.KATZ, L.HK] * 8, seeds[:24], eps[:24],
                            alphas=[0.1, 1.0 / (float(g.degree.max()) + 1.0), 0.0] * 8, tau=5.0, prec="fp64",
                            slots=6, tuning={"groups": groups})
    ref = api.serve_mixed(Gd, [L.PPR, L.KATZ, L.HK] * 8, seeds[:24], eps[:24],
                          alphas=[0.1, 1.0 / (float(g.degree.max()) + 1.0), 0.0] * 8, tau=5.0, prec="fp64",
                          slots=6, tuning={"groups": 1})
    np.testing.assert_allclose(mixed["oper"], ref["oper"], rtol=1e-12)
    for i in range(24):
        assert rel_l1(mixed["x"][i], ref["x"][i]) < FP64_L1, i


def test_rows_into_pinned_device_and_pageable_memory_agree(cl):
    """Pinned host rows are written by the device directly; device rows in place;
    pageable rows through staging.  All three hold the same values (Katz seed
    correction and heat-kernel scale included)."""
    import torch
    g, Gd = cl
    nq = 30
    kinds = np.array([L.PPR, L.KATZ, L.HK] * (nq // 3), dtype=np.int32)
    seeds = graphs.uniform_seeds(g, nq, seed=27)
    eps = np.exp(np.random.default_rng(27).uniform(np.log(1e-6), np.log(1e-5), nq))
    alphas = np.where(kinds == L.KATZ, 1.0 / (float(g.degree.max()) + 1.0), 0.1)
    kw = dict(alphas=alphas, tau=5.0, prec="fp32", slots=3)
    pinned = torch.full((nq, g.n), float("nan"), dtype=torch.float32).pin_memory()
    a = api.serve_mixed(Gd, kinds, seeds, eps, x_out=pinned, device_out=False, **kw)
    dev = torch.full((nq, g.n), float("nan"), dtype=torch.float32, device="cuda")
    b = api.serve_mixed(Gd, kinds, seeds, eps, x_out=dev, device_out=True, **kw)
    c = api.serve_mixed(Gd, kinds, seeds, eps, **kw)  # pageable numpy rows
    xb = dev.cpu().numpy()
    assert np.isfinite(pinned.numpy()).all() and np.isfinite(xb).all()
    for i in range(nq):
        alone = (api.solve(Gd, L.HK, L.HK_LOCAL, seeds[i:i + 1], eps[i:i + 1], prec="fp64", tau=5.0, want_r=False)
                 if kinds[i] == L.HK else
                 api.solve(Gd, int(kinds[i]), L.LOCAL_GD, seeds[i:i + 1], eps[i:i + 1], prec="fp64",
                           alpha=float(alphas[i]), tile_w=1, want_r=False))
        for x in (pinned[i].numpy(), xb[i], c["x"][i]):
            assert rel_l1(x, alone["x"][0]) < 1e-4, (i, int(kinds[i]))
    np.testing.assert_allclose(a["oper"], b["oper"], rtol=1e-3)
