"""ctypes front-end of the C restatement in ``gde_oracle.c`` (test infrastructure only).

The C file restates the reference's solvers (``ppr_solver.py``,
``katz_solver.py``, ``hk_solver.py``, ``InstantGNN.py``) in FP64 with the same
floating-point operation order; these wrappers take and return numpy arrays
in the reference's calling convention.  ``build()`` compiles the library with
gcc (``-ffp-contract=off`` so no FMA changes a rounding, OpenMP for the timed
multi-query baseline).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "gde_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgde_oracle.so")

_lib = None
_lib_lock = threading.Lock()  # the first call may come from several worker threads at once
_i64 = ctypes.c_int64
_dbl = ctypes.c_double
_int = ctypes.c_int
_p = ctypes.c_void_p


def build(force: bool = False) -> str:
    """Compile ``gde_oracle.c`` into ``_build/libgde_oracle.so`` (skipped when up to date)."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + f".{os.getpid()}.{threading.get_ident()}.tmp"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c99", SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def lib():
    with _lib_lock:
        return _lib if _lib is not None else _load()


def _load():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.orc_ppr_gd.restype = _i64
        L.orc_ppr_gd.argtypes = [_i64, _p, _p, _p, _i64, _dbl, _dbl, _int, _p, _p]
        L.orc_cheby.restype = _i64
        L.orc_cheby.argtypes = [_i64, _p, _p, _p, _i64, _dbl, _dbl, _int, _int, _dbl, _dbl, _int, _p, _p]
        L.orc_katz_gd.restype = _i64
        L.orc_katz_gd.argtypes = [_i64, _p, _p, _p, _i64, _dbl, _dbl, _int, _p, _p]
        L.orc_sor.restype = _dbl
        L.orc_sor.argtypes = [_i64, _p, _p, _p, _i64, _dbl, _dbl, _dbl, _int, _int, _p, _p]
        L.orc_ign_sor_color_column.restype = _i64
        L.orc_ign_sor_color_column.argtypes = [_i64, _p, _p, _p, _dbl, _p, _dbl, _dbl, _p, _p, _i64, _p, _p, _i64,
                                               _int]
        L.orc_sor_color.restype = _dbl
        L.orc_sor_color.argtypes = [_i64, _p, _p, _p, _i64, _dbl, _dbl, _dbl, _int, _int, _p, _i64, _p, _p, _p]
        L.orc_hk_estimate_n.restype = _i64
        L.orc_hk_estimate_n.argtypes = [_dbl, _dbl]
        L.orc_hk_sor_queue.restype = _dbl
        L.orc_hk_sor_queue.argtypes = [_i64, _p, _p, _p, _i64, _dbl, _dbl, _dbl, _int, _p, _p, _p]
        L.orc_hk_sor_sync.restype = _dbl
        L.orc_hk_sor_sync.argtypes = [_i64, _p, _p, _p, _i64, _dbl, _dbl, _dbl, _int, _p, _p, _p]
        L.orc_hk_taylor.restype = _i64
        L.orc_hk_taylor.argtypes = [_i64, _p, _p, _p, _i64, _dbl, _dbl, _p]
        L.orc_ign_static_column.restype = _i64
        L.orc_ign_static_column.argtypes = [_i64, _p, _p, _p, _dbl, _dbl, _dbl, _int, _dbl, _p, _i64, _p, _i64]
        L.orc_update_graph.restype = None
        L.orc_update_graph.argtypes = [_i64, _p, _p, _p, _p, _p, _i64, _int, _p, _p, _p, _p, _p, _p, _p, _p]
        L.orc_ign_update_column.restype = _i64
        L.orc_ign_update_column.argtypes = [_i64, _p, _p, _p, _p, _p, _p, _p, _i64, _dbl, _dbl, _dbl, _int, _int,
                                            _dbl, _p, _p, _p, _i64, _p, _p, _p, _i64, _int, _p, _i64]
        L.orc_update_ppr_row.restype = _i64
        L.orc_update_ppr_row.argtypes = [_i64, _p, _p, _p, _p, _p, _p, _dbl, _dbl, _dbl, _p, _p, _p, _i64, _p, _p,
                                         _p, _i64, _int, _p, _i64]
        L.orc_ign_sync_column.restype = _i64
        L.orc_ign_sync_column.argtypes = [_i64, _p, _p, _p, _dbl, _dbl, _p, _dbl, _p, _p, _i64, _p, _i64]
        L.orc_threads.restype = _int
        L.orc_ppr_gd_many.restype = None
        L.orc_ppr_gd_many.argtypes = [_i64, _p, _p, _p, _p, _i64, _dbl, _p, _int, _p, _p, _int]
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _graph(indptr, indices, degree):
    indptr = np.ascontiguousarray(indptr, dtype=np.int64)
    indices = np.ascontiguousarray(indices, dtype=np.int32)
    degree = np.ascontiguousarray(degree, dtype=np.float64)
    return indptr, indices, degree


def ppr_gd(n, indptr, indices, degree, s, alpha, eps, local):
    """``ppr_solver.ppr_gd`` (ppr_solver.py:208-328) -> (x, r, oper)."""
    indptr, indices, degree = _graph(indptr, indices, degree)
    x = np.zeros(n)
    r = np.zeros(n)
    oper = lib().orc_ppr_gd(n, _ptr(indptr), _ptr(indices), _ptr(degree), int(s), alpha, eps, int(local), _ptr(x),
                            _ptr(r))
    return x, r, int(oper)


def cheby(n, indptr, indices, degree, s, alpha, eps, local, katz=False, l_max=0.0, mu_min=0.0, sync=False):
    """``ppr_cheby`` (ppr_solver.py:582-661) / ``katz_cheby`` (katz_solver.py:340-431) -> (x, r, oper)."""
    indptr, indices, degree = _graph(indptr, indices, degree)
    x = np.zeros(n)
    r = np.zeros(n)
    oper = lib().orc_cheby(n, _ptr(indptr), _ptr(indices), _ptr(degree), int(s), alpha, eps, int(local), int(katz),
                           l_max, mu_min, int(sync), _ptr(x), _ptr(r))
    return x, r, int(oper)


def katz_gd(n, indptr, indices, degree, s, alpha, eps, local):
    """``katz_solver.katz_gd`` (katz_solver.py:167-248) -> (x, r, oper)."""
    indptr, indices, degree = _graph(indptr, indices, degree)
    x = np.zeros(n)
    r = np.zeros(n)
    oper = lib().orc_katz_gd(n, _ptr(indptr), _ptr(indices), _ptr(degree), int(s), alpha, eps, int(local), _ptr(x),
                             _ptr(r))
    return x, r, int(oper)


def sor(n, indptr, indices, degree, s, alpha, eps, omega, local, katz=False):
    """``ppr_sor`` (ppr_solver.py:331-461) / ``katz_sor`` (katz_solver.py:251-337) -> (x, r, oper)."""
    indptr, indices, degree = _graph(indptr, indices, degree)
    x = np.zeros(n)
    r = np.zeros(n)
    oper = lib().orc_sor(n, _ptr(indptr), _ptr(indices), _ptr(degree), int(s), alpha, eps, omega, int(local),
                         int(katz), _ptr(x), _ptr(r))
    return x, r, float(oper)


def sor_color(n, indptr, indices, degree, s, alpha, eps, omega, local, colors, katz=False):
    """Multicolour local/global SOR (the GPU LocalSOR order) -> (x, r, oper, sweeps)."""
    indptr, indices, degree = _graph(indptr, indices, degree)
    colors = np.ascontiguousarray(colors, dtype=np.int32)
    x = np.zeros(n)
    r = np.zeros(n)
    sw = ctypes.c_int64()
    oper = lib().orc_sor_color(n, _ptr(indptr), _ptr(indices), _ptr(degree), int(s), alpha, eps, omega, int(local),
                               int(katz), _ptr(colors), int(colors.max()) + 1 if colors.size else 0, _ptr(x), _ptr(r),
                               ctypes.byref(sw))
    return x, r, float(oper), int(sw.value)


def greedy_colors(indptr, indices, order, row_len=None):
    """Greedy proper colouring visiting nodes in ``order`` (smallest colour not used by a coloured neighbour).

    ``row_len`` gives the used length of each row of a padded CSR.
    """
    n = len(indptr) - 1
    ends = indptr[1:] if row_len is None else indptr[:-1] + row_len
    col = np.full(n, -1, dtype=np.int32)
    for u in order:
        used = {int(col[v]) for v in indices[indptr[u]:ends[u]] if col[v] >= 0}
        c = 0
        while c in used:
            c += 1
        col[u] = c
    return col


def hk_estimate_n(t, eps):
    """``hk_solver.estimate_n`` (hk_solver.py:28-48)."""
    return int(lib().orc_hk_estimate_n(t, eps))


def hk_sor_queue(n, indptr, indices, degree, s, tau, eps, omega, local, sync=False):
    """``hk_solver.hk_sor_queue`` (hk_solver.py:206-295) -> (est_n, x, r[2,n], oper).

    sync=True: the level-synchronous form (every node at or above threshold
    relaxes at its level, no re-enqueue test on the next level's mark); equal
    to the reference for omega = 1 and for the global form.
    """
    indptr, indices, degree = _graph(indptr, indices, degree)
    x = np.zeros(n)
    r = np.zeros((2, n))
    est = np.zeros(1, dtype=np.int64)
    fn = lib().orc_hk_sor_sync if sync else lib().orc_hk_sor_queue
    oper = fn(n, _ptr(indptr), _ptr(indices), _ptr(degree), int(s), tau, eps, omega, int(local), _ptr(x), _ptr(r),
              _ptr(est))
    return int(est[0]), x, r, float(oper)


def hk_taylor(n, indptr, indices, degree, s, tau, eps):
    """``hk_solver.hk_taylor_approx`` (hk_solver.py:51-80) -> (est_n, x)."""
    indptr, indices, degree = _graph(indptr, indices, degree)
    x = np.zeros(n)
    est = lib().orc_hk_taylor(n, _ptr(indptr), _ptr(indices), _ptr(degree), int(s), tau, eps, _ptr(x))
    return int(est), x


def _ign_graph(indptr, indices, degree):
    return (np.ascontiguousarray(indptr, dtype=np.int64), np.ascontiguousarray(indices, dtype=np.int32),
            np.ascontiguousarray(degree, dtype=np.int64))


def ign_static(n, indptr, indices, degree, alpha, eps, P, R, beta, omega=1.0, sor=False):
    """``instantGNNParallel`` / ``instantGNNSorParallel`` (InstantGNN.py:46-134); P, R (n x F) in place.

    Returns the per-column work of the FIFO push (sum of the pushing nodes' degrees; the reference
    itself returns only run times).
    """
    indptr, indices, degree = _ign_graph(indptr, indices, degree)
    assert P.dtype == np.float64 and R.dtype == np.float64 and P.flags.c_contiguous and R.flags.c_contiguous
    F = R.shape[1]
    opers = np.zeros(F, np.int64)
    for f in range(F):
        opers[f] = lib().orc_ign_static_column(n, _ptr(indptr), _ptr(indices), _ptr(degree), alpha, eps, omega,
                                               int(sor), beta, P.ctypes.data + 8 * f, F, R.ctypes.data + 8 * f, F)
    return opers


def update_graph(n, indptr, indices, degree, us, vs, onlyinsert):
    """``updetaGraph`` (InstantGNN.py:137-180); mutates indices/degree in place.

    Returns (ins_keys, ins_off, ins_nbr, del_keys, del_off, del_nbr).
    """
    k = len(us)
    us = np.ascontiguousarray(us, dtype=np.int64)
    vs = np.ascontiguousarray(vs, dtype=np.int64)
    assert indices.dtype == np.int32 and degree.dtype == np.int64 and indptr.dtype == np.int64
    ik = np.zeros(2 * k + 1, np.int64)
    io = np.zeros(2 * k + 2, np.int64)
    inb = np.zeros(2 * k + 1, np.int64)
    dk = np.zeros(2 * k + 1, np.int64)
    do = np.zeros(2 * k + 2, np.int64)
    dnb = np.zeros(2 * k + 1, np.int64)
    ni = np.zeros(1, np.int64)
    nd = np.zeros(1, np.int64)
    lib().orc_update_graph(n, _ptr(indptr), _ptr(indices), _ptr(degree), _ptr(us), _ptr(vs), k, int(onlyinsert),
                           _ptr(ik), _ptr(io), _ptr(inb), _ptr(ni), _ptr(dk), _ptr(do), _ptr(dnb), _ptr(nd))
    a, b = int(ni[0]), int(nd[0])
    return ik[:a], io[:a + 1], inb[:io[a]], dk[:b], do[:b + 1], dnb[:do[b]]


def _padded_colors(indptr, indices, degree):
    """The GPU's colouring of a padded graph: greedy in degree-descending order, ties by id."""
    return greedy_colors(indptr, indices, np.argsort(-degree, kind="stable"), row_len=degree)


def ign_update(n, indptr, indices, degree, alpha, eps, omega, P, R, X, us, vs, beta, algo, sync=False, color=False):
    """``instantGNNUpdateBatchParallel`` (InstantGNN.py:332-359); mutates graph, P, R in place.

    sync=True keeps the reference's repair and uses the synchronous push;
    color=True keeps it and relaxes in multicolour SOR order (colouring of the
    edited graph); returns (maps, per-column push opers).
    """
    old_degree = degree.copy()
    maps = update_graph(n, indptr, indices, degree, us, vs, "insert" in algo)
    mode = 2 if color else (1 if sync else 0)
    col = _padded_colors(indptr, indices, degree) if color else np.zeros(1, np.int32)
    ik, io, inb, dk, do, dnb = maps
    F = R.shape[1]
    X = np.ascontiguousarray(X, dtype=np.float64)
    opers = np.zeros(F, np.int64)

    def column(f):
        opers[f] = lib().orc_ign_update_column(n, _ptr(indptr), _ptr(indices), _ptr(degree), _ptr(old_degree),
                                               P.ctypes.data + 8 * f, R.ctypes.data + 8 * f, X.ctypes.data + 8 * f, F,
                                               alpha, eps, omega, int("sor" in algo), int("insert" in algo), beta,
                                               _ptr(ik), _ptr(io), _ptr(inb), len(ik), _ptr(dk), _ptr(do), _ptr(dnb),
                                               len(dk), mode, _ptr(col), int(col.max()) + 1)
    _columns(F, column)
    return maps, opers


def update_ppr(n, indptr, indices, degree, alpha, eps, omega, P, R, us, vs, sync=False, color=False):
    """``update_ppr_parallel`` (ppr_solver.py:824-849); P, R are F x n, updated in place -> opers.

    sync=True keeps the reference's repair and uses the synchronous push;
    color=True keeps it and relaxes in multicolour SOR order.
    """
    old_degree = degree.copy()
    ik, io, inb, dk, do, dnb = update_graph(n, indptr, indices, degree, us, vs, False)
    mode = 2 if color else (1 if sync else 0)
    col = _padded_colors(indptr, indices, degree) if color else np.zeros(1, np.int32)
    opers = np.zeros(P.shape[0], np.int64)
    for f in range(P.shape[0]):
        p = np.ascontiguousarray(P[f])
        r = np.ascontiguousarray(R[f])
        opers[f] = lib().orc_update_ppr_row(n, _ptr(indptr), _ptr(indices), _ptr(degree), _ptr(old_degree), _ptr(p),
                                            _ptr(r), alpha, eps, omega, _ptr(ik), _ptr(io), _ptr(inb), len(ik),
                                            _ptr(dk), _ptr(do), _ptr(dnb), len(dk), mode, _ptr(col),
                                            int(col.max()) + 1)
        P[f] = p
        R[f] = r
    return opers


def ign_sync(n, indptr, indices, degree, alpha, eps, beta, P, R, cand0=None, max_rounds=1 << 30, x_gain=None):
    """Synchronous InstantGNN push (the GPU's frontier rule) on every column of P, R in place.

    Returns per-column operation counts.
    """
    indptr, indices, degree = _ign_graph(indptr, indices, degree)
    eps_vec = np.power(degree.astype(np.float64), 1 - beta) * eps
    F = R.shape[1]
    if cand0 is None:
        cand0 = np.ones(n, np.uint8)
    cand0 = np.ascontiguousarray(cand0, dtype=np.uint8)
    opers = np.zeros(F, np.int64)

    def column(f):
        opers[f] = lib().orc_ign_sync_column(n, _ptr(indptr), _ptr(indices), _ptr(degree), alpha,
                                             alpha if x_gain is None else x_gain, _ptr(eps_vec), beta,
                                             P.ctypes.data + 8 * f, R.ctypes.data + 8 * f, F, _ptr(cand0), max_rounds)
    _columns(F, column)
    return opers


def ign_sor_color(n, indptr, indices, degree, alpha, eps, beta, omega, P, R, colors, cand0=None):
    """Multicolour SOR InstantGNN push (the GPU order) on every column of P, R in place -> opers."""
    indptr, indices, degree = _ign_graph(indptr, indices, degree)
    eps_vec = np.power(degree.astype(np.float64), 1 - beta) * eps
    F = R.shape[1]
    if cand0 is None:
        cand0 = np.ones(n, np.uint8)
    cand0 = np.ascontiguousarray(cand0, dtype=np.uint8)
    colors = np.ascontiguousarray(colors, dtype=np.int32)
    opers = np.zeros(F, np.int64)
    for f in range(F):
        opers[f] = lib().orc_ign_sor_color_column(n, _ptr(indptr), _ptr(indices), _ptr(degree), alpha,
                                                  _ptr(eps_vec), beta, omega, P.ctypes.data + 8 * f,
                                                  R.ctypes.data + 8 * f, F, _ptr(cand0), _ptr(colors),
                                                  int(colors.max()) + 1, 0)
    return opers


def _columns(F: int, fn) -> None:
    """fn(f) for every column f, on host threads (each column's C call touches only its own column of P, R;
    ctypes releases the GIL around the call)."""
    if F <= 1:
        for f in range(F):
            fn(f)
        return
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=min(F, os.cpu_count() or 1)) as ex:
        list(ex.map(fn, range(F)))


def threads() -> int:
    return int(lib().orc_threads())


def ppr_gd_many(n, indptr, indices, degree, seeds, alpha, eps, local=True, keep_x=False, nthreads=0):
    """Many PPR local-GD queries, one per OpenMP thread (the timed CPU baseline)."""
    indptr, indices, degree = _graph(indptr, indices, degree)
    seeds = np.ascontiguousarray(seeds, dtype=np.int64)
    eps = np.ascontiguousarray(np.broadcast_to(np.asarray(eps, np.float64), seeds.shape))
    oper = np.zeros(seeds.shape[0], np.int64)
    x = np.zeros((seeds.shape[0], n)) if keep_x else None
    lib().orc_ppr_gd_many(n, _ptr(indptr), _ptr(indices), _ptr(degree), _ptr(seeds), seeds.shape[0], alpha, _ptr(eps),
                          int(local), _ptr(oper), _ptr(x) if keep_x else None, int(nthreads))
    return oper, x


def global_solve_ppr(indptr, indices, degree, s, alpha, tol=1e-15, max_iter=100000):
    """FP64 truth: x = alpha (I - (1-alpha) A D^-1)^-1 e_s by Jacobi iteration to ||r||_1 < tol."""
    import scipy.sparse as sp
    n = len(indptr) - 1
    A = sp.csr_matrix((np.ones(len(indices)), indices, indptr), shape=(n, n))
    M = (A @ sp.diags(1.0 / np.asarray(degree, np.float64))).tocsr() * (1.0 - alpha)
    r = np.zeros(n)
    r[s] = alpha
    x = np.zeros(n)
    for _ in range(max_iter):
        x += r
        r = M @ r
        if np.abs(r).sum() < tol:
            break
    return x + r
