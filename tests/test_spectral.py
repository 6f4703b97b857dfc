"""Katz Chebyshev spectral bounds by GPU Lanczos against scipy's eigsh.

The reference's experiment scripts take lambda_max(A) (eigsh which='LM')
and lambda_min(A) (which='SA') of the adjacency (katz_exp_dmax.py:20,
katz_exp_dmin.py:20); the GPU Lanczos must agree, and the bounds it gives
must make katz_cheby converge to the Katz solution.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

from gde import _lib as L
from gde import api, graphs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", ["cl", "rmat"])
def test_lanczos_extremes_match_eigsh(which):
    if which == "cl":
        g = graphs.chung_lu(3000, 2.1, 8.0, 300.0, seed=3)
    else:
        g = graphs.rmat(12, 16, 0.57, 0.19, 0.19, seed=1)
    A = sp.csr_matrix((np.ones(g.nnz), g.indices, g.indptr), shape=(g.n, g.n))
    lmax = sla.eigsh(A, 1, which="LA", tol=1e-12)[0][0]
    lmin = sla.eigsh(A, 1, which="SA", tol=1e-12)[0][0]
    Gd = api.Graph(g.indptr, g.indices)
    alpha = 0.5 / lmax
    b = api.katz_spectral_bounds(Gd, alpha, tol=1e-11)
    assert b["lam_max"] == pytest.approx(lmax, rel=1e-8)
    assert b["lam_min"] == pytest.approx(lmin, rel=1e-7, abs=1e-7 * lmax)
    assert b["l_max"] == pytest.approx(1 - alpha * lmin, rel=1e-8)
    assert b["mu_min"] == pytest.approx(1 - alpha * lmax, rel=1e-8)


def test_bounds_drive_katz_cheby():
    g = graphs.chung_lu(3000, 2.1, 8.0, 300.0, seed=3)
    Gd = api.Graph(g.indptr, g.indices)
    b = api.katz_spectral_bounds(Gd, 1.0)  # lambdas only
    alpha = 0.5 / b["lam_max"]
    l_max, mu_min = 1 - alpha * b["lam_min"], 1 - alpha * b["lam_max"]
    s = int(graphs.uniform_seeds(g, 1, seed=5)[0])
    res = api.solve(Gd, L.KATZ, L.GLOBAL_CHEBY, [s], [1e-9], prec="fp64", alpha=alpha, l_max=l_max, mu_min=mu_min)
    # FP64 truth: (I - alpha A) x = e_s
    A = sp.csr_matrix((np.ones(g.nnz), g.indices, g.indptr), shape=(g.n, g.n))
    e = np.zeros(g.n)
    e[s] = 1.0
    truth = sla.spsolve((sp.identity(g.n) - alpha * A).tocsc(), e)
    assert np.abs(res["x"][0] - truth).sum() / np.abs(truth).sum() < 1e-6
    # and the same bounds as the oracle's Chebyshev takes them
    xo, _, _ = O.cheby(g.n, g.indptr, g.indices, g.degree.astype(np.float64), s, alpha, 1e-9, False, katz=True,
                       l_max=l_max, mu_min=mu_min, sync=True)
    assert np.abs(res["x"][0] - xo).sum() / np.abs(xo).sum() < 1e-10


@pytest.mark.gpu
def test_katz_near_its_radius_computes_in_fp64():
    """An FP32 Katz request with alpha * lambda_max >= 0.9 is computed in FP64 (gde_stats.prec),
    and then follows the FP64 solve's trajectory: the same operation counts and solutions.

    Near the radius a trajectory is near-critical: a threshold test that an FP64 rounding of the
    atomics' order flips can change the rest of the run, so one of the seeds may diverge between
    two FP64 runs; the others must agree exactly.
    """
    from gde import _lib as L
    from gde import api, graphs
    g = graphs.chung_lu(3000, 2.1, 8.0, 300.0, seed=12)
    Gd = api.Graph(g.indptr, g.indices)
    lam = api.katz_spectral_bounds(Gd, 0.01)["lam_max"]
    seeds = graphs.uniform_seeds(g, 6, seed=3)
    alpha = 0.95 / lam
    for tile_w in (1, 4):
        r32 = api.solve(Gd, L.KATZ, L.LOCAL_GD, seeds, 1e-6, prec="fp32", alpha=alpha, tile_w=tile_w)
        r64 = api.solve(Gd, L.KATZ, L.LOCAL_GD, seeds, 1e-6, prec="fp64", alpha=alpha, tile_w=tile_w)
        assert r32["stats"]["prec"] == L.FP64 and r64["stats"]["prec"] == L.FP64
        assert r32["x"].dtype == np.float32  # the rows keep the requested format
        same = r32["oper"] == r64["oper"]
        assert same.sum() >= len(seeds) - 1, (r32["oper"], r64["oper"])
        for i in np.nonzero(same)[0]:
            ref = r64["x"][i]
            assert np.abs(r32["x"][i].astype(np.float64) - ref).sum() <= 1e-6 * np.abs(ref).sum()
    # a fresh graph object (no cached estimate) decides the same way, through its own Lanczos run
    G2 = api.Graph(g.indptr, g.indices)
    r = api.solve(G2, L.KATZ, L.LOCAL_GD, seeds, 1e-6, prec="fp32", alpha=alpha, tile_w=1)
    assert r["stats"]["prec"] == L.FP64
    # far from the radius an FP32 request stays in FP32
    r = api.solve(Gd, L.KATZ, L.LOCAL_GD, seeds, 1e-6, prec="fp32", alpha=0.5 / lam, tile_w=1)
    assert r["stats"]["prec"] == L.FP32
