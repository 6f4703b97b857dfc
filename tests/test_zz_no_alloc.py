"""The allocation-free single-query solve (gde_solve_noalloc) against gde_solve.

gde_solve_noalloc runs the push engine out of a fixed device array inside the
library.  Each case calls it twice in a row through the C ABI (the second call
reuses the array the first one left behind) and compares both results with
the existing entry point, gde_solve, on the same query at the same precision:
FP64 within the FP64 tolerance of the parity tests and with the same
operation counts, FP32 within the FP32 tolerance.  This file is collected last so
that it also runs after every other GPU test in the same process.
"""
import ctypes

import numpy as np
import pytest

from gde import _lib as L
from gde import api, graphs

pytestmark = pytest.mark.gpu

FP64_L1 = 1e-12      # relative l1 of FP64 solutions (same bar as the parity tests)
FP32_L1 = 2e-6       # relative l1 between FP32 solutions, plus a few threshold flips (below)
OPER_RTOL = 1e-12


@pytest.fixture(scope="module")
def cl():
    g = graphs.chung_lu(3000, 2.1, 8.0, 300.0, seed=3)
    return g, api.Graph(g.indptr, g.indices)


def rel_l1(a, b):
    return np.abs(np.asarray(a, np.float64) - b).sum() / max(np.abs(b).sum(), 1e-300)


def noalloc(Gd, kind, method, seed, eps, prec, alpha):
    import torch
    lib = L.load()
    out64 = prec == "fp64"
    dt = torch.float64 if out64 else torch.float32
    x = torch.full((Gd.n,), float("nan"), dtype=dt, device=f"cuda:{Gd.ctx.device}")
    r = torch.full((Gd.n,), float("nan"), dtype=dt, device=f"cuda:{Gd.ctx.device}")
    torch.cuda.synchronize()
    p = api.make_params(kind, method, prec=prec, alpha=alpha)
    oper = ctypes.c_double()
    rounds = ctypes.c_int32()
    st = lib.gde_solve_noalloc(Gd.ctx.ptr, Gd.ptr, ctypes.byref(p), int(seed), float(eps), x.data_ptr(),
                               r.data_ptr(), int(out64), ctypes.byref(oper), ctypes.byref(rounds))
    L.check(Gd.ctx.ptr, st, "gde_solve_noalloc")
    return x.cpu().numpy(), r.cpu().numpy(), oper.value, rounds.value


def existing(Gd, kind, method, seed, eps, prec, alpha):
    res = api.solve(Gd, kind, method, [int(seed)], [eps], prec=prec, alpha=alpha)
    return res["x"][0], res["r"][0], res["oper"][0], int(res["rounds"][0])


CASES = [
    ("ppr-local", L.PPR, L.LOCAL_GD, 0.15, 1e-6),
    ("ppr-global", L.PPR, L.GLOBAL_GD, 0.15, 1e-5),
    ("katz-local", L.KATZ, L.LOCAL_GD, None, 1e-6),
]


@pytest.mark.parametrize("name,kind,method,alpha,eps", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_noalloc_matches_gde_solve_twice(cl, name, kind, method, alpha, eps, prec):
    g, Gd = cl
    if alpha is None:
        alpha = 1.0 / (float(g.degree.max()) + 1.0)   # below 1 / lambda_max
    seeds = graphs.uniform_seeds(g, 2, seed=11)
    for call in range(2):
        s = int(seeds[call])
        xe, re_, oe, ke = existing(Gd, kind, method, s, eps, prec, alpha)
        x, r, o, k = noalloc(Gd, kind, method, s, eps, prec, alpha)
        assert np.isfinite(x).all() and np.isfinite(r).all(), (name, call)
        if prec == "fp64":
            assert o == pytest.approx(oe, rel=OPER_RTOL), (name, call, o, oe)
            assert k == ke, (name, call)
            assert rel_l1(x, xe) < FP64_L1, (name, call)
            assert np.abs(r - re_).sum() < 1e-12 * max(np.abs(re_).sum(), 1.0), (name, call)
        else:
            # two FP32 runs add residuals in different orders, so a node within
            # rounding of its threshold may push a round apart in the two: each
            # such flip moves about 2*theta*d_u of mass (sum(x) ~ 1)
            theta = eps * (alpha if kind == L.PPR else 1.0)
            flips = 3 * 2 * theta * float(g.degree.max())
            assert rel_l1(x, xe) < FP32_L1 + flips, (name, call, rel_l1(x, xe))
            # FP32 residuals can flip a threshold tie: opers agree to a few edges
            assert abs(o - oe) <= 1e-3 * oe, (name, call, o, oe)


def test_noalloc_katz_near_its_radius_keeps_the_fp64_rule(cl):
    """An FP32 Katz query with alpha * lambda_max >= 0.9 computes in FP64 in both entry points.

    The largest degree cannot clear it here, so on a graph without a spectral
    estimate the allocation-free call computes in FP64 (its operation counts
    are the FP64 solve's); once the estimate is cached, gde_solve and the
    allocation-free call take the same precision and agree to the FP64 bar,
    twice in a row.
    """
    g, _ = cl
    fresh = api.Graph(g.indptr, g.indices)      # no spectral estimate cached yet
    lam = api.katz_spectral_bounds(api.Graph(g.indptr, g.indices), 0.1)["lam_max"]
    alpha = 0.95 / lam
    assert alpha * float(g.degree.max()) >= 0.9
    seeds = graphs.uniform_seeds(g, 2, seed=12)
    _, _, o64, _ = existing(fresh, L.KATZ, L.LOCAL_GD, int(seeds[0]), 1e-6, "fp64", alpha)
    _, _, o, _ = noalloc(fresh, L.KATZ, L.LOCAL_GD, int(seeds[0]), 1e-6, "fp32", alpha)
    assert o == pytest.approx(o64, rel=OPER_RTOL)
    api.katz_spectral_bounds(fresh, alpha)      # caches the estimate gde_solve would compute
    for call in range(2):
        s = int(seeds[call])
        xe, re_, oe, ke = existing(fresh, L.KATZ, L.LOCAL_GD, s, 1e-6, "fp32", alpha)
        x, r, o, k = noalloc(fresh, L.KATZ, L.LOCAL_GD, s, 1e-6, "fp32", alpha)
        assert o == pytest.approx(oe, rel=OPER_RTOL), (call, o, oe)
        assert k == ke
        # both computed in FP64 and rounded to FP32 rows
        assert rel_l1(x, xe.astype(np.float64)) < 1e-6, call
    fresh.free()


def test_noalloc_rejects_graph_above_the_fixed_scratch():
    n = 2_000_000                    # ~90 MB of FP32 workspace > the 64 MiB array
    u = np.arange(n - 1, dtype=np.int64)
    g, _ = graphs._csr_from_undirected(n, u, u + 1, drop_isolated=False)   # a path
    Gd = api.Graph(g.indptr, g.indices)
    with pytest.raises(L.GDEError) as ei:
        noalloc(Gd, L.PPR, L.LOCAL_GD, 0, 1e-4, "fp32", 0.15)
    assert ei.value.status == L.GDE_EINVAL
    assert "fixed scratch" in str(ei.value)
    Gd.free()
