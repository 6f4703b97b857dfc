"""Generate the golden fixtures in this directory by running the reference itself.

The reference solvers are numba-compiled Python (``ppr_solver.py``,
``katz_solver.py``, ``hk_solver.py``, ``InstantGNN.py``).  numba, cupy and
torch_sparse are not installed here, so this script installs small stand-in
modules (``njit`` = identity, ``objmode`` = no-op context manager, ``prange`` =
``range``, typed ``List``/``Dict`` = Python ``list``/``dict``) and then imports
and runs the reference's *own* CPU code, unmodified, as plain Python.  Two
behaviours of plain Python differ from numba and are bridged here:

* ``estimate_n`` (``hk_solver.py:37-42``) passes a float to ``range``; numba
  accepts it, Python does not.  The module's ``range`` is replaced by one that
  truncates float arguments to int, as numba does.
* integer degree arrays are passed (float degrees break the row slicing
  ``indices[indptr[u]:indptr[u]+degree[u]]`` of ``ppr_sor``/InstantGNN).
* ``instantGNNUpdateBatchParallel`` allocates an ``n+1`` queue but wraps it
  modulo ``n+2`` (``InstantGNN.py:316``, ``:344``), so compiled numba (no bounds
  checks) writes and later reads back one slot past the end.  numpy raises
  instead, so InstantGNN's ``np.zeros`` is given one spare slot for 1-D integer
  arrays, which reproduces what the compiled code reads back.

Usage:  python tests/golden/make_golden.py /path/to/reference
Writes ``tests/golden/golden_*.npz``.  The fixtures are small (graphs of a few
hundred nodes) so the whole script runs in a few minutes.
"""
from __future__ import annotations

import builtins
import contextlib
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "faster-local-solver-for-gdes_gb300"))

from gde import graphs  # noqa: E402


def install_shims() -> None:
    numba = types.ModuleType("numba")

    def njit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    @contextlib.contextmanager
    def objmode(**kwargs):
        yield

    class _T:
        int64 = "int64"
        int32 = "int32"
        float64 = "float64"

        @staticmethod
        def ListType(t):
            return ("list", t)

    class List(list):
        @staticmethod
        def empty_list(t):
            return []

    class Dict(dict):
        @staticmethod
        def empty(key_type=None, value_type=None):
            return {}

    typed = types.ModuleType("numba.typed")
    typed.List = List
    typed.Dict = Dict
    numba.njit = njit
    numba.jit = njit
    numba.vectorize = njit
    numba.objmode = objmode
    numba.prange = range
    numba.types = _T
    numba.typed = typed
    numba.cuda = types.ModuleType("numba.cuda")
    sys.modules["numba"] = numba
    sys.modules["numba.typed"] = typed
    sys.modules["numba.cuda"] = numba.cuda
    cupy = types.ModuleType("cupy")
    cupy.ndarray = type("ndarray", (), {})  # scipy's array-API probe looks this up
    sys.modules["cupy"] = cupy
    sys.modules["torch_sparse"] = types.ModuleType("torch_sparse")


def _int_range(*args):
    return builtins.range(*[int(a) for a in args])


class _PaddedNumpy:
    """numpy facade whose ``zeros`` adds one spare slot to 1-D integer arrays."""

    def __getattr__(self, name):
        return getattr(np, name)

    @staticmethod
    def zeros(shape, dtype=float, **kw):
        if isinstance(shape, (int, np.integer)) and np.issubdtype(np.dtype(dtype), np.integer):
            return np.zeros(int(shape) + 1, dtype=dtype, **kw)
        return np.zeros(shape, dtype=dtype, **kw)


def small_graphs() -> dict[str, graphs.CSRGraph]:
    gs = {}
    gs["cl300"] = graphs.chung_lu(300, 2.1, 6.0, 60.0, seed=11)
    gs["cl800"] = graphs.chung_lu(800, 2.3, 8.0, 120.0, seed=12)
    # star with a tail (hub + degree-1 leaves) and a clique joined to a path
    n = 40
    a = [0] * 30 + list(range(30, 39))
    b = list(range(1, 31)) + list(range(31, 40))
    gs["star_tail"], _ = graphs._csr_from_undirected(n, np.array(a), np.array(b), True)
    k = 12
    aa, bb = [], []
    for i in range(k):
        for j in range(i + 1, k):
            aa.append(i)
            bb.append(j)
    for i in range(k - 1, k + 10):
        aa.append(i)
        bb.append(i + 1)
    gs["clique_path"], _ = graphs._csr_from_undirected(k + 11, np.array(aa), np.array(bb), True)
    return gs


def spectral_bounds(g: graphs.CSRGraph) -> tuple[float, float]:
    import scipy.sparse as sp
    from scipy.sparse.linalg import eigsh
    A = sp.csr_matrix((np.ones(g.nnz), g.indices, g.indptr), shape=(g.n, g.n))
    lam_max = float(abs(eigsh(A, 1, which="LM")[0][0]))
    lam_min = float(eigsh(A, 1, which="SA")[0][0])
    return lam_max, lam_min


def main(ref: str) -> None:
    install_shims()
    sys.path.insert(0, ref)
    import ppr_solver
    import katz_solver
    import hk_solver
    import InstantGNN
    hk_solver.range = _int_range
    InstantGNN.np = _PaddedNumpy()

    out = {}
    gs = small_graphs()
    for gname, g in gs.items():
        out[f"graph/{gname}/indptr"] = g.indptr
        out[f"graph/{gname}/indices"] = g.indices
    case = 0

    def put(kind, gname, params, **arrays):
        nonlocal case
        key = f"case{case:03d}"
        out[key + "/kind"] = np.array(kind)
        out[key + "/graph"] = np.array(gname)
        for k, v in params.items():
            out[key + "/p/" + k] = np.array(v)
        for k, v in arrays.items():
            out[key + "/o/" + k] = np.array(v, copy=True)  # solvers mutate P, R, indices in place
        case += 1

    # --- PPR: ppr_gd local/global, ppr_cheby local/global, ppr_sor (ppr_solver.py:208-661)
    for gname, g in gs.items():
        deg = g.degree
        rng = np.random.default_rng(5)
        seeds = rng.integers(0, g.n, size=3)
        for s in seeds:
            for alpha, eps in [(0.1, 1e-4), (0.2, 1e-6)] if g.n >= 300 else [(0.15, 1e-5)]:
                for local in (True, False):
                    x, r, oper, _ = ppr_solver.ppr_gd(g.n, g.indptr, g.indices, deg, int(s), alpha, eps, local, None)
                    put("ppr_gd", gname, dict(s=int(s), alpha=alpha, eps=eps, local=local), x=x, r=r, oper=oper)
                    x, r, oper, _ = ppr_solver.ppr_cheby(g.n, g.indptr, g.indices, deg, int(s), alpha, eps, local)
                    put("ppr_cheby", gname, dict(s=int(s), alpha=alpha, eps=eps, local=local), x=x, r=r, oper=oper)
                    for omega in (1.0, 1.2):
                        x, r, oper, _ = ppr_solver.ppr_sor(g.n, g.indptr, g.indices, deg, int(s), alpha, eps, omega, local, None)
                        put("ppr_sor", gname, dict(s=int(s), alpha=alpha, eps=eps, omega=omega, local=local),
                            x=x, r=r, oper=oper)

    # --- Katz: katz_gd, katz_cheby, katz_sor (katz_solver.py:167-431)
    for gname, g in gs.items():
        deg = g.degree
        lam_max, lam_min = spectral_bounds(g)
        alpha = 0.5 / lam_max
        l_max = 1.0 - alpha * lam_min
        mu_min = 1.0 - alpha * lam_max
        rng = np.random.default_rng(6)
        for s in rng.integers(0, g.n, size=2):
            for eps in (1e-5, 1e-7):
                for local in (True, False):
                    x, r, oper, _ = katz_solver.katz_gd(g.n, g.indptr, g.indices, deg, int(s), alpha, eps, local)
                    put("katz_gd", gname, dict(s=int(s), alpha=alpha, eps=eps, local=local), x=x, r=r, oper=oper)
                    x, r, oper, _ = katz_solver.katz_cheby(g.n, g.indptr, g.indices, deg, int(s), alpha, l_max, mu_min,
                                                           eps, local)
                    put("katz_cheby", gname, dict(s=int(s), alpha=alpha, eps=eps, local=local, l_max=l_max,
                                                  mu_min=mu_min), x=x, r=r, oper=oper)
                    x, r, oper, _ = katz_solver.katz_sor(g.n, g.indptr, g.indices, deg, int(s), alpha, eps, 1.1, local)
                    put("katz_sor", gname, dict(s=int(s), alpha=alpha, eps=eps, omega=1.1, local=local),
                        x=x, r=r, oper=oper)

    # --- Heat kernel: estimate_n, hk_taylor_approx, hk_sor_queue (hk_solver.py:15-295)
    for t, e in [(1.0, 1e-3), (3.0, 1e-6), (5.0, 1e-4), (5.0, 1e-8), (10.0, 1e-7), (2.5, 0.3)]:
        put("estimate_n", "", dict(tau=t, eps=e), n=int(hk_solver.estimate_n(t, e)))
    for gname, g in gs.items():
        deg = g.degree
        rng = np.random.default_rng(7)
        for s in rng.integers(0, g.n, size=2):
            for tau, eps in [(5.0, 1e-5), (3.0, 1e-7)]:
                for local in (True, False):
                    for omega in (1.0,) if not local else (1.0, 1.3):
                        est_n, x, r, oper, beta_t, _, _ = hk_solver.hk_sor_queue(
                            g.n, g.indptr, g.indices, deg, int(s), tau, eps, omega, local)
                        put("hk_sor_queue", gname, dict(s=int(s), tau=tau, eps=eps, omega=omega, local=local),
                            est_n=int(est_n), x=x, r=r, oper=oper)
                est_n, x, _ = hk_solver.hk_taylor_approx(g.n, g.indptr, g.indices, deg, int(s), tau, eps)
                put("hk_taylor_approx", gname, dict(s=int(s), tau=tau, eps=eps), est_n=int(est_n), x=x)

    # --- InstantGNN (InstantGNN.py:12-359) and dynamic PPR update (ppr_solver.py:723-849)
    base = graphs.chung_lu(400, 2.3, 10.0, 80.0, seed=13, drop_isolated=False)
    dg = graphs.dynamic_padded(base, 900, 3, seed=14)
    out["dyn/indptr"] = dg.indptr
    out["dyn/indices"] = dg.indices
    out["dyn/degree"] = dg.degree
    out["dyn/Us"] = dg.Us
    out["dyn/Vs"] = dg.Vs
    F = 6
    rng = np.random.default_rng(15)
    X = rng.standard_normal((dg.n, F))
    out["dyn/X"] = X
    alpha, eps, beta = 0.1, 1e-4, 0.5
    a2 = alpha / (2 - alpha)
    mu = (1. - a2) / (1. + a2)
    omega = 1. + (mu / (1. + np.sqrt(1. - mu ** 2.))) ** 2.
    for algo in ("fwdbatchinsert", "sorbatchinsert", "fwdbatch"):
        indptr = dg.indptr.copy()
        indices = dg.indices.copy()
        degree = dg.degree.copy()
        P = np.zeros((dg.n, F))
        R = X.copy()
        if algo.startswith("sor"):
            InstantGNN.instantGNNSorParallel(dg.n, indptr, indices, degree, alpha, eps, omega, P, R, beta, batchsize=4)
        else:
            InstantGNN.instantGNNParallel(dg.n, indptr, indices, degree, alpha, eps, P, R, beta, batchsize=4)
        put("instantgnn_static", "dyn", dict(algo=algo, alpha=alpha, eps=eps, beta=beta, omega=omega), P=P, R=R)
        for snap in range(dg.Us.shape[0]):
            us = dg.Us[snap].copy()
            vs = dg.Vs[snap].copy()
            if algo == "fwdbatch" and snap == 2:
                # a batch that re-sends half of the edges just inserted: with a
                # non-insert algo these become deletions (InstantGNN.py:151-168)
                us = np.concatenate([dg.Us[1][: len(us) // 2], us[len(us) // 2:]])
                vs = np.concatenate([dg.Vs[1][: len(vs) // 2], vs[len(vs) // 2:]])
            InstantGNN.instantGNNUpdateBatchParallel(dg.n, indptr, indices, degree, alpha, eps, omega, P, R, X,
                                                     us, vs, beta, algo, batchsize=4)
            put("instantgnn_update", "dyn", dict(algo=algo, alpha=alpha, eps=eps, beta=beta, omega=omega, snap=snap),
                us=us, vs=vs, P=P, R=R, indices=indices, degree=degree)
    # update_ppr_parallel: P, R are F x n (one row per feature), beta = 0 form
    indptr = dg.indptr.copy()
    indices = dg.indices.copy()
    degree = dg.degree.copy()
    Fp = 3
    P = np.zeros((Fp, dg.n))
    R = np.zeros((Fp, dg.n))
    seeds = rng.integers(0, dg.n, size=Fp)
    for f, s in enumerate(seeds):
        R[f, s] = alpha
    out["dynppr/seeds"] = seeds
    for snap in range(2):
        opers, _, P, R = ppr_solver.update_ppr_parallel(dg.n, indptr, indices, degree, alpha, 1e-4, 1.0, P, R,
                                                        dg.Us[snap].astype(np.int64), dg.Vs[snap].astype(np.int64),
                                                        batchsize=2)
        put("update_ppr", "dyn", dict(alpha=alpha, eps=1e-4, omega=1.0, snap=snap), opers=opers, P=P.copy(),
            R=R.copy(), indices=indices.copy(), degree=degree.copy())

    path = os.path.join(HERE, "golden_reference.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {case} cases to {path} ({os.path.getsize(path) / 1e6:.2f} MB)")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GDE_REFERENCE", "reference"))
