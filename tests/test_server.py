"""Online serving (gde_server_*): queries submitted while the persistent launch runs.

The server's kernel admits queries from a ring in pinned host memory at
round boundaries.  These tests submit queries while earlier ones are on the
GPU (one launch serves them all), and check that every result equals the same
query solved alone through gde_solve: FP64 operation counts exactly and
solutions to 1e-12, for PPR, Katz and heat-kernel queries mixed in one
stream; FP32 rows within the FP32 bound.  They also cover the stop flag (a
clean exit, with and without draining), the idle exit and relaunch, and the
argument checks.
"""
import time

import numpy as np
import pytest

from gde import _lib as L
from gde import api, graphs

pytestmark = pytest.mark.gpu

TAU = 5.0


@pytest.fixture(scope="module")
def cl():
    g = graphs.chung_lu(3000, 2.1, 8.0, 300.0, seed=3)
    return g, api.Graph(g.indptr, g.indices)


def _queries(g, k, seed):
    rng = np.random.default_rng(seed)
    kinds = rng.choice([L.PPR, L.KATZ, L.HK], size=k, p=[0.5, 0.25, 0.25])
    seeds = graphs.uniform_seeds(g, k, seed=seed)
    eps = np.exp(rng.uniform(np.log(1e-7), np.log(1e-5), k))
    alphas = np.where(kinds == L.KATZ, 0.5 / float(g.degree.max()), 0.15)
    return kinds, seeds, eps, alphas


def _alone(Gd, kind, s, eps, alpha, prec):
    if kind == L.HK:
        r = api.solve(Gd, L.HK, L.HK_LOCAL, [int(s)], [eps], prec=prec, tau=TAU, want_r=False)
    else:
        r = api.solve(Gd, int(kind), L.LOCAL_GD, [int(s)], [eps], prec=prec, alpha=float(alpha), want_r=False,
                      tile_w=1)
    return r["x"][0], r["oper"][0]


def _wait(srv, tickets, timeout_s=60.0):
    out = {}
    t0 = time.time()
    while len(out) < len(tickets):
        for t in tickets:
            if t not in out:
                r = srv.poll(t)
                if r is not None:
                    out[t] = r
        assert time.time() - t0 < timeout_s, "queries did not finish"
    return out


@pytest.mark.parametrize("slots,groups", [(4, 0), (8, 4), (6, 6)])
def test_submissions_while_running_equal_the_query_alone(cl, slots, groups):
    """Queries submitted while earlier ones run, in one launch: each equals the query alone.  With
    several slot groups, group 0 places requests into the idle slots of every group, and each group
    admits them at its own round boundary behind its own barrier."""
    import torch
    g, Gd = cl
    srv = api.Server(Gd, prec="fp64", slots=slots, tau=TAU, idle_ms=500.0,
                     tuning={"groups": groups} if groups else None)
    kinds, seeds, eps, alphas = _queries(g, 16, seed=41)
    rows = torch.full((16, g.n), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    tickets = [srv.submit(kinds[i], seeds[i], eps[i], alphas[i], rows[i], out64=True) for i in range(6)]
    # the rest arrive while the first ones are on the GPU
    _wait(srv, tickets[:1])
    tickets += [srv.submit(kinds[i], seeds[i], eps[i], alphas[i], rows[i], out64=True) for i in range(6, 16)]
    res = _wait(srv, tickets)
    info = srv.info()
    assert srv.stop(drain=True) == 0
    assert info["launches"] == 1, info  # one launch admitted every query
    x = rows.cpu().numpy()
    for i, t in enumerate(tickets):
        xa, oa = _alone(Gd, kinds[i], seeds[i], eps[i], alphas[i], "fp64")
        assert res[t]["oper"] == pytest.approx(oa, rel=1e-12), (i, kinds[i])
        assert np.abs(x[i] - xa).sum() <= 1e-12 * np.abs(xa).sum(), (i, kinds[i])
        assert res[t]["device_ms"] > 0


def test_fp32_server_into_pinned_host_rows(cl):
    import torch
    g, Gd = cl
    srv = api.Server(Gd, prec="fp32", slots=8, tau=TAU, idle_ms=50.0)
    kinds, seeds, eps, alphas = _queries(g, 12, seed=42)
    rows = [torch.full((g.n,), float("nan"), dtype=torch.float32).pin_memory() for _ in range(12)]
    tickets = [srv.submit(kinds[i], seeds[i], eps[i], alphas[i], rows[i]) for i in range(12)]
    res = _wait(srv, tickets)
    srv.stop()
    for i, t in enumerate(tickets):
        xa, oa = _alone(Gd, kinds[i], seeds[i], eps[i], alphas[i], "fp32")
        x = rows[i].numpy()
        assert np.isfinite(x).all()
        # two FP32 runs add residuals in different orders: a node within rounding
        # of its threshold may push a round apart (2 theta d of l1 each)
        theta = eps[i] * (0.15 if kinds[i] == L.PPR else 1.0)
        bound = 2e-6 * max(np.abs(xa).sum(), 1.0) + 3 * 2 * theta * float(g.degree.max()) * (
            np.exp(TAU) if kinds[i] == L.HK else 1.0)
        assert np.abs(x.astype(np.float64) - xa).sum() < bound, (i, kinds[i])
        assert abs(res[t]["oper"] - oa) <= 1e-3 * oa + 64, (i, res[t]["oper"], oa)


def test_idle_exit_then_relaunch_on_the_next_submit(cl):
    import torch
    g, Gd = cl
    srv = api.Server(Gd, prec="fp64", slots=2, idle_ms=1.0)
    seeds = graphs.uniform_seeds(g, 4, seed=43)
    rows = torch.zeros((4, g.n), dtype=torch.float64, device="cuda")
    t0 = [srv.submit(L.PPR, seeds[i], 1e-6, 0.15, rows[i], out64=True) for i in range(2)]
    _wait(srv, t0)
    time.sleep(0.2)  # the kernel leaves after 1 ms idle
    t1 = [srv.submit(L.PPR, seeds[i], 1e-6, 0.15, rows[i], out64=True) for i in range(2, 4)]
    res = _wait(srv, t1)
    info = srv.info()
    srv.stop()
    assert info["launches"] >= 2, info
    x = rows.cpu().numpy()
    for i in range(4):
        xa, oa = _alone(Gd, L.PPR, seeds[i], 1e-6, 0.15, "fp64")
        assert np.abs(x[i] - xa).sum() <= 1e-12
    for i, t in enumerate(t1):
        assert res[t]["oper"] == pytest.approx(_alone(Gd, L.PPR, seeds[2 + i], 1e-6, 0.15, "fp64")[1], rel=1e-12)


def test_stop_flag_ends_the_kernel_cleanly(cl):
    import torch
    g, Gd = cl
    srv = api.Server(Gd, prec="fp64", slots=2, idle_ms=10_000.0)
    assert srv.stop(drain=False) == 0  # nothing submitted
    srv = api.Server(Gd, prec="fp64", slots=2, idle_ms=10_000.0)
    seeds = graphs.uniform_seeds(g, 6, seed=44)
    rows = torch.zeros((6, g.n), dtype=torch.float64, device="cuda")
    for i in range(6):
        srv.submit(L.PPR, seeds[i], 1e-8, 0.01, rows[i], out64=True)
    lost = srv.stop(drain=False)  # the kernel leaves at its next round; unfinished queries are dropped
    assert 0 <= lost <= 6
    # the device and the context are fine afterwards
    srv = api.Server(Gd, prec="fp64", slots=2, idle_ms=5.0)
    t = srv.submit(L.PPR, seeds[0], 1e-6, 0.15, rows[0], out64=True)
    res = _wait(srv, [t])
    srv.stop()
    assert res[t]["oper"] == pytest.approx(_alone(Gd, L.PPR, seeds[0], 1e-6, 0.15, "fp64")[1], rel=1e-12)


def test_submit_checks(cl):
    import torch
    g, Gd = cl
    srv = api.Server(Gd, prec="fp32", slots=2, idle_ms=5.0)
    try:
        hub = int(np.argmax(g.degree))
        with pytest.raises(L.GDEError) as ei:
            srv.submit(L.PPR, hub, 1.0, 0.15)  # eps * degree[s] > 1 (ppr_solver.py:213)
        assert ei.value.status == L.GDE_EINVAL
        with pytest.raises(L.GDEError) as ei:
            srv.submit(L.HK, 0, 1e-6)  # no tau given at start
        assert ei.value.status == L.GDE_EINVAL
        with pytest.raises(L.GDEError) as ei:  # Katz near its radius needs FP64
            srv.submit(L.KATZ, 0, 1e-6, 0.95 / float(g.degree.max()))
        assert ei.value.status == L.GDE_EINVAL
        with pytest.raises(L.GDEError) as ei:  # pageable host memory is not device-addressable
            srv.submit(L.PPR, 0, 1e-6, 0.15, torch.zeros(g.n, dtype=torch.float32))
        assert ei.value.status == L.GDE_EINVAL
        with pytest.raises(L.GDEError) as ei:
            srv.poll(10_000)
        assert ei.value.status == L.GDE_ENOTFOUND
    finally:
        srv.stop()
