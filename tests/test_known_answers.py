"""Known answers on tiny graphs: path, star, clique, lollipop.

Every push solver keeps an exact linear identity between its solution and
residual, so on a graph small enough for a direct solve (scipy ``spsolve``)
the answer is known in closed form:

* PPR (``ppr_solver.py:208-328``, ``:582-661``): with Q = I - (1-alpha) A D^-1,
  every push keeps ``Q x + r = alpha e_s``, so ``x + Q^-1 r`` is the exact PPR
  vector and ``sum(x) + sum(r) / alpha = 1`` (A D^-1 is column-stochastic).
* Katz (``katz_solver.py:167-248``): with Q = I - alpha A the push keeps
  ``Q (x + e_s) + r = e_s`` (the reference subtracts e_s at the end).
* Heat kernel (``hk_solver.py:51-80``): the Taylor sum of exp(-tau (I - A D^-1))
  e_s, compared with ``scipy.sparse.linalg.expm_multiply``.

At exit local GD also meets its stopping rule ``|r_u| < eps alpha d_u``.  The
CPU tests pin the oracle; the GPU tests hold the library's FP64 and FP32
paths to the same identities.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle import oracle as O


def _csr(n, edges):
    a = np.array([e[0] for e in edges] + [e[1] for e in edges], np.int64)
    b = np.array([e[1] for e in edges] + [e[0] for e in edges], np.int64)
    A = sp.csr_matrix((np.ones(a.size), (a, b)), shape=(n, n))
    A.sum_duplicates()
    A.sort_indices()
    return A.indptr.astype(np.int64), A.indices.astype(np.int32), np.diff(A.indptr).astype(np.int64)


def _graphs():
    path = _csr(12, [(i, i + 1) for i in range(11)])
    star = _csr(21, [(0, i) for i in range(1, 21)])
    clique = _csr(10, [(i, j) for i in range(10) for j in range(i + 1, 10)])
    lolli = _csr(12, [(i, j) for i in range(6) for j in range(i + 1, 6)] + [(i, i + 1) for i in range(5, 11)])
    return {"path": path, "star": star, "clique": clique, "lollipop": lolli}


GRAPHS = _graphs()
CASES = [(name, s) for name in GRAPHS for s in (0, len(GRAPHS[name][2]) - 1)]


def _adj(ip, ix):
    n = len(ip) - 1
    return sp.csr_matrix((np.ones(len(ix)), ix, ip), shape=(n, n))


def ppr_q(ip, ix, deg, alpha):
    A = _adj(ip, ix)
    return (sp.identity(A.shape[0]) - (1 - alpha) * (A @ sp.diags(1.0 / deg))).tocsc()


def katz_q(ip, ix, alpha):
    A = _adj(ip, ix)
    return (sp.identity(A.shape[0]) - alpha * A).tocsc()


def ppr_truth(ip, ix, deg, s, alpha):
    b = np.zeros(len(deg))
    b[s] = alpha
    return spla.spsolve(ppr_q(ip, ix, deg, alpha), b)


def katz_alpha(deg):
    return 0.5 / float(deg.max())


def check_ppr_identity(ip, ix, deg, s, alpha, x, r, tol):
    """x + Q^-1 r equals the exact PPR vector; the mass identity holds."""
    truth = ppr_truth(ip, ix, deg, s, alpha)
    rec = x + spla.spsolve(ppr_q(ip, ix, deg, alpha), r)
    assert np.abs(rec - truth).sum() < tol
    assert abs(x.sum() + r.sum() / alpha - 1.0) < tol


def check_katz_identity(ip, ix, s, alpha, x, r, tol):
    n = len(ip) - 1
    Q = katz_q(ip, ix, alpha)
    e = np.zeros(n)
    e[s] = 1.0
    truth = spla.spsolve(Q, e) - e
    rec = x + spla.spsolve(Q, r)
    assert np.abs(rec - truth).sum() < tol * max(1.0, np.abs(truth).sum())


def hk_truth(ip, ix, deg, s, tau):
    A = _adj(ip, ix)
    L = (A @ sp.diags(1.0 / deg)) - sp.identity(A.shape[0])
    e = np.zeros(A.shape[0])
    e[s] = 1.0
    return spla.expm_multiply(tau * L.tocsc(), e)


# ----------------------------------------------------------------- oracle (CPU)

@pytest.mark.parametrize("name,s", CASES)
@pytest.mark.parametrize("local", [True, False])
def test_oracle_ppr_gd_identity(name, s, local):
    ip, ix, deg = GRAPHS[name]
    alpha, eps = 0.15, 1e-7
    x, r, _ = O.ppr_gd(len(deg), ip, ix, deg, s, alpha, eps, local)
    check_ppr_identity(ip, ix, deg, s, alpha, x, r, 1e-12)
    if local:
        assert (np.abs(r) < eps * alpha * deg).all()
    # and the solution is within the residual's reach of the truth
    assert np.abs(x - ppr_truth(ip, ix, deg, s, alpha)).sum() <= np.abs(r).sum() / alpha + 1e-12


@pytest.mark.parametrize("name,s", CASES)
def test_oracle_ppr_cheby_identity(name, s):
    ip, ix, deg = GRAPHS[name]
    alpha, eps = 0.15, 1e-7
    x, r, _ = O.cheby(len(deg), ip, ix, deg, s, alpha, eps, True)
    check_ppr_identity(ip, ix, deg, s, alpha, x, r, 1e-12)


@pytest.mark.parametrize("name,s", CASES)
@pytest.mark.parametrize("local", [True, False])
def test_oracle_katz_gd_identity(name, s, local):
    ip, ix, deg = GRAPHS[name]
    alpha = katz_alpha(deg)
    x, r, _ = O.katz_gd(len(deg), ip, ix, deg, s, alpha, 1e-8, local)
    check_katz_identity(ip, ix, s, alpha, x, r, 1e-12)


@pytest.mark.parametrize("name,s", CASES)
def test_oracle_hk_taylor_matches_expm(name, s):
    ip, ix, deg = GRAPHS[name]
    tau, eps = 3.0, 1e-8
    _, x = O.hk_taylor(len(deg), ip, ix, deg, s, tau, eps)
    assert np.abs(x - hk_truth(ip, ix, deg, s, tau)).sum() < 1e-7


# ----------------------------------------------------------------- GPU

def _gpu_graph(name):
    from gde import api
    ip, ix, deg = GRAPHS[name]
    return api.Graph(ip, ix)


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(GRAPHS))
def test_gpu_ppr_identities(name):
    from gde import _lib as L
    from gde import api
    ip, ix, deg = GRAPHS[name]
    G = _gpu_graph(name)
    alpha, eps = 0.15, 1e-7
    seeds = [0, len(deg) - 1]
    for method in (L.LOCAL_GD, L.GLOBAL_GD, L.LOCAL_CHEBY, L.GLOBAL_CHEBY):
        res = api.solve(G, L.PPR, method, seeds, eps, prec="fp64", alpha=alpha, tile_w=1)
        for i, s in enumerate(seeds):
            check_ppr_identity(ip, ix, deg, s, alpha, res["x"][i], res["r"][i], 1e-12)
            if method == L.LOCAL_GD:
                assert (np.abs(res["r"][i]) < eps * alpha * deg).all()
    # FP32 residuals, Kahan FP32 solution: the identities to FP32 rounding
    res = api.solve(G, L.PPR, L.LOCAL_GD, seeds, eps, prec="fp32", alpha=alpha, tile_w=1)
    for i, s in enumerate(seeds):
        x = res["x"][i].astype(np.float64)
        r = res["r"][i].astype(np.float64)
        check_ppr_identity(ip, ix, deg, s, alpha, x, r, 1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(GRAPHS))
def test_gpu_served_ppr_identity(name):
    from gde import _lib as L
    from gde import api
    ip, ix, deg = GRAPHS[name]
    G = _gpu_graph(name)
    alpha, eps = 0.15, 1e-7
    seeds = np.arange(len(deg), dtype=np.int32)
    res = api.serve(G, L.PPR, seeds, eps, alpha=alpha, prec="fp32", want_r=False, slots=4)
    for i, s in enumerate(seeds):
        truth = ppr_truth(ip, ix, deg, int(s), alpha)
        # |x - x*|_1 <= |r|_1 / alpha < eps * vol: the local-push guarantee, plus FP32 rounding
        assert np.abs(res["x"][i].astype(np.float64) - truth).sum() < eps * deg.sum() + 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(GRAPHS))
def test_gpu_katz_identity(name):
    from gde import _lib as L
    from gde import api
    ip, ix, deg = GRAPHS[name]
    G = _gpu_graph(name)
    alpha = katz_alpha(deg)
    seeds = [0, len(deg) - 1]
    for method in (L.LOCAL_GD, L.GLOBAL_GD):
        res = api.solve(G, L.KATZ, method, seeds, 1e-8, prec="fp64", alpha=alpha, tile_w=1)
        for i, s in enumerate(seeds):
            check_katz_identity(ip, ix, s, alpha, res["x"][i], res["r"][i], 1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(GRAPHS))
def test_gpu_hk_taylor_matches_expm(name):
    from gde import _lib as L
    from gde import api
    ip, ix, deg = GRAPHS[name]
    G = _gpu_graph(name)
    tau, eps = 3.0, 1e-8
    seeds = [0, len(deg) - 1]
    res = api.solve(G, L.HK, L.HK_TAYLOR, seeds, eps, prec="fp64", tau=tau, want_r=False, tile_w=1)
    for i, s in enumerate(seeds):
        assert np.abs(res["x"][i] - hk_truth(ip, ix, deg, s, tau)).sum() < 1e-7
