"""Python host API over the C ABI: contexts, resident graphs, batched solves.

This is the layer the drop-in modules (``ppr_solver``, ``katz_solver``,
``hk_solver``, ``InstantGNN``) and the benchmark call.  Device buffers are
torch tensors (plumbing only); every solver runs in ``libgde.so``.
"""
from __future__ import annotations

import ctypes
import weakref

import numpy as np

from . import _lib as L

_PREC = {"fp64": L.FP64, "fp32": L.FP32}


def _ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch tensor


class Context:
    """One CUDA device + stream + workspace of the library (``gde_ctx``)."""

    _by_device: dict[int, "Context"] = {}

    def __init__(self, device: int = 0):
        lib = L.load()
        h = ctypes.c_void_p()
        st = lib.gde_ctx_create(device, ctypes.byref(h))
        if st != L.GDE_OK:
            raise L.GDEError(st, f"gde_ctx_create(device={device}) failed: {lib.gde_status_str(st).decode()}")
        self.ptr = h.value
        self.device = device
        self._fin = weakref.finalize(self, lib.gde_ctx_destroy, h.value)

    @classmethod
    def get(cls, device: int = 0) -> "Context":
        c = cls._by_device.get(device)
        if c is None:
            c = cls._by_device[device] = Context(device)
        return c

    def close(self) -> None:
        self._fin()


class Graph:
    """A CSR graph resident in device memory (``gde_graph``).

    ``row_len`` = live entries per row (padded InstantGNN CSR); default is the
    row-pointer difference.  ``degree`` = arithmetic degree used in the
    formulas; default is the row length.
    """

    def __init__(self, indptr, indices, row_len=None, degree=None, ctx: Context | None = None):
        self.ctx = ctx or Context.get(0)
        lib = L.load()
        indptr = np.ascontiguousarray(indptr, dtype=np.int64)
        indices = np.ascontiguousarray(indices, dtype=np.int32)
        n = indptr.shape[0] - 1
        rl = None if row_len is None else np.ascontiguousarray(row_len, dtype=np.int64)
        dg = None if degree is None else np.ascontiguousarray(degree, dtype=np.float64)
        h = ctypes.c_void_p()
        st = lib.gde_graph_upload(self.ctx.ptr, n, indices.shape[0], _ptr(indptr), _ptr(indices), _ptr(rl), _ptr(dg),
                                  ctypes.byref(h))
        L.check(self.ctx.ptr, st, "gde_graph_upload")
        self.ptr = h.value
        self.n = int(n)
        self.cap = int(indices.shape[0])
        vol = ctypes.c_double()
        lib.gde_graph_info(self.ptr, None, None, ctypes.byref(vol))
        self.vol = float(vol.value)
        self._fin = weakref.finalize(self, lib.gde_graph_free, h.value)

    def free(self) -> None:
        self._fin()


def make_params(kind: int, method: int, prec: str = "fp64", tile_w: int = 0, alpha: float = 0.0, tau: float = 0.0,
                l_max: float = 0.0, mu_min: float = 0.0, beta: float = 0.0, omega: float = 1.0, max_rounds: int = 0,
                tuning: dict | None = None) -> L.Params:
    p = L.Params()
    p.kind, p.method, p.prec, p.tile_w = kind, method, _PREC[prec], tile_w
    p.alpha, p.tau, p.l_max, p.mu_min, p.beta, p.omega = alpha, tau, l_max, mu_min, beta, omega
    p.max_rounds = max_rounds
    t = tuning or {}
    p.small_max = int(t.get("small_max", 0))
    p.med_max = int(t.get("med_max", 0))
    p.chunk = int(t.get("chunk", 0))
    p.dense_div = int(t.get("dense_div", 0))
    p.slots = int(t.get("slots", 0))
    p.groups = int(t.get("groups", 0))
    # served small queries out of hash tables: {"sparse_blocks": B, "sparse_eps": e, "sparse_cap": C}
    p.sparse_blocks = int(t.get("sparse_blocks", 0))
    p.sparse_cap = int(t.get("sparse_cap", 0))
    p.sparse_eps = float(t.get("sparse_eps", 0.0))
    return p


def solve(graph: Graph, kind: int, method: int, seeds, eps, *, prec: str = "fp64", out64: bool | None = None,
          want_x: bool = True, want_r: bool = True, x_out=None, r_out=None, device_out: bool = False,
          tile_w: int = 0, alpha: float = 0.0, tau: float = 0.0, l_max: float = 0.0, mu_min: float = 0.0,
          max_rounds: int = 0, tuning: dict | None = None, omega: float = 1.0) -> dict:
    """Solve one query per seed; returns dict(x, r, oper, rounds, stats).

    ``omega`` (heat-kernel level push only): relaxation of hk_sor_queue, in (0, 2).

    ``x_out`` / ``r_out`` may be caller buffers (numpy / torch, host or
    device per ``device_out``) of shape [nq, n] (HK residual: [nq, 2, n]).
    """
    lib = L.load()
    seeds = np.ascontiguousarray(np.atleast_1d(seeds), dtype=np.int32)
    nq = seeds.shape[0]
    eps = np.ascontiguousarray(np.broadcast_to(np.asarray(eps, dtype=np.float64), (nq,)))
    if out64 is None:
        out64 = prec == "fp64"
    n = graph.n
    rl = 2 if (kind == L.HK and method != L.HK_TAYLOR) else 1
    odt = np.float64 if out64 else np.float32
    if want_x and x_out is None:
        if device_out:
            import torch
            x_out = torch.empty((nq, n), dtype=torch.float64 if out64 else torch.float32,
                                device=f"cuda:{graph.ctx.device}")
        else:
            x_out = np.empty((nq, n), dtype=odt)
    if want_r and r_out is None:
        shape = (nq, rl, n) if rl == 2 else (nq, n)
        if device_out:
            import torch
            r_out = torch.empty(shape, dtype=torch.float64 if out64 else torch.float32,
                                device=f"cuda:{graph.ctx.device}")
        else:
            r_out = np.empty(shape, dtype=odt)
    oper = np.zeros(nq, dtype=np.float64)
    rounds = np.zeros(nq, dtype=np.int32)
    lat = np.zeros(nq, dtype=np.float32)
    p = make_params(kind, method, prec, tile_w, alpha, tau, l_max, mu_min, omega=omega, max_rounds=max_rounds,
                    tuning=tuning)
    st = L.Stats()
    status = lib.gde_solve(graph.ctx.ptr, graph.ptr, ctypes.byref(p), nq, _ptr(seeds), _ptr(eps),
                           _ptr(x_out) if want_x else None, _ptr(r_out) if want_r else None, int(out64),
                           L.MEM_DEVICE if device_out else L.MEM_HOST, n, _ptr(oper), _ptr(rounds), _ptr(lat),
                           ctypes.byref(st))
    L.check(graph.ctx.ptr, status, "gde_solve")
    return {"x": x_out if want_x else None, "r": r_out if want_r else None, "oper": oper, "rounds": rounds,
            "latency_ms": lat, "stats": st.as_dict()}


def serve(graph: Graph, kind: int, seeds, eps, *, arrival_ms=None, prec: str = "fp32", out64: bool | None = None,
          want_x: bool = True, want_r: bool = False, x_out=None, r_out=None, device_out: bool = False,
          alpha: float = 0.0, slots: int = 0, max_rounds: int = 0, tuning: dict | None = None) -> dict:
    """Served PPR / Katz local GD (continuous batching); returns dict(x, r, oper, rounds, latency_ms, stats).

    ``arrival_ms[q]``: query q arrives that many ms after the launch starts
    and its latency is measured from its arrival (None: all at time 0).
    """
    lib = L.load()
    seeds = np.ascontiguousarray(np.atleast_1d(seeds), dtype=np.int32)
    nq = seeds.shape[0]
    eps = np.ascontiguousarray(np.broadcast_to(np.asarray(eps, dtype=np.float64), (nq,)))
    arr = None if arrival_ms is None else np.ascontiguousarray(arrival_ms, dtype=np.float64)
    if out64 is None:
        out64 = prec == "fp64"
    n = graph.n
    if want_x and x_out is None:
        x_out = _alloc((nq, n), out64, device_out, graph)
    if want_r and r_out is None:
        r_out = _alloc((nq, n), out64, device_out, graph)
    oper = np.zeros(nq, dtype=np.float64)
    rounds = np.zeros(nq, dtype=np.int32)
    lat = np.zeros(nq, dtype=np.float32)
    t = dict(tuning or {})
    if slots:
        t["slots"] = slots
    p = make_params(kind, L.LOCAL_GD, prec, 1, alpha, max_rounds=max_rounds, tuning=t)
    st = L.Stats()
    status = lib.gde_serve(graph.ctx.ptr, graph.ptr, ctypes.byref(p), nq, _ptr(seeds), _ptr(eps), _ptr(arr),
                           _ptr(x_out) if want_x else None, _ptr(r_out) if want_r else None, int(out64),
                           L.MEM_DEVICE if device_out else L.MEM_HOST, n, _ptr(oper), _ptr(rounds), _ptr(lat),
                           ctypes.byref(st))
    L.check(graph.ctx.ptr, status, "gde_serve")
    return {"x": x_out if want_x else None, "r": r_out if want_r else None, "oper": oper, "rounds": rounds,
            "latency_ms": lat, "stats": st.as_dict()}


def serve_mixed(graph: Graph, kinds, seeds, eps, *, alphas=None, tau: float = 0.0, arrival_ms=None,
                hbm_budget_bytes: float = 0.0, prec: str = "fp32", out64: bool | None = None, want_x: bool = True,
                x_out=None, device_out: bool = False, slots: int = 0, max_rounds: int = 0,
                tuning: dict | None = None) -> dict:
    """Served mix of PPR / Katz / heat-kernel queries (continuous batching, one persistent launch).

    ``kinds[q]`` in (L.PPR, L.KATZ, L.HK); ``alphas[q]`` for PPR / Katz; heat
    kernel uses ``tau``.  Returns dict(x, oper, rounds, latency_ms, stats).
    """
    lib = L.load()
    kinds = np.ascontiguousarray(np.atleast_1d(kinds), dtype=np.int32)
    seeds = np.ascontiguousarray(np.atleast_1d(seeds), dtype=np.int32)
    nq = seeds.shape[0]
    eps = np.ascontiguousarray(np.broadcast_to(np.asarray(eps, dtype=np.float64), (nq,)))
    al = None if alphas is None else np.ascontiguousarray(np.broadcast_to(np.asarray(alphas, np.float64), (nq,)))
    arr = None if arrival_ms is None else np.ascontiguousarray(arrival_ms, dtype=np.float64)
    if out64 is None:
        out64 = prec == "fp64"
    n = graph.n
    if want_x and x_out is None:
        x_out = _alloc((nq, n), out64, device_out, graph)
    oper = np.zeros(nq, dtype=np.float64)
    rounds = np.zeros(nq, dtype=np.int32)
    lat = np.zeros(nq, dtype=np.float32)
    t = dict(tuning or {})
    if slots:
        t["slots"] = slots
    p = make_params(L.PPR, L.LOCAL_GD, prec, 1, 0.0, tau, max_rounds=max_rounds, tuning=t)
    st = L.Stats()
    status = lib.gde_serve_mixed(graph.ctx.ptr, graph.ptr, ctypes.byref(p), nq, _ptr(kinds), _ptr(seeds), _ptr(eps),
                                 _ptr(al), _ptr(arr), float(hbm_budget_bytes), _ptr(x_out) if want_x else None,
                                 int(out64), L.MEM_DEVICE if device_out else L.MEM_HOST, n, _ptr(oper), _ptr(rounds),
                                 _ptr(lat), ctypes.byref(st))
    L.check(graph.ctx.ptr, status, "gde_serve_mixed")
    return {"x": x_out if want_x else None, "oper": oper, "rounds": rounds, "latency_ms": lat, "stats": st.as_dict()}


class Server:
    """Online serving (``gde_server_*``): queries submitted while one persistent launch runs.

    ``submit`` returns a ticket; ``poll(ticket)`` returns None until the
    query's row is written, then dict(oper, rounds, device_ms).  Rows go into
    the caller's buffer: a device tensor or a pinned host tensor of n entries
    (float32, or float64 with out64).  ``stop(drain=True)`` waits for every
    submitted query, then ends the kernel and frees the server.
    """

    def __init__(self, graph: Graph, *, prec: str = "fp32", slots: int = 0, tau: float = 0.0,
                 ring_capacity: int = 4096, hbm_budget_bytes: float = 0.0, idle_ms: float = 5.0,
                 tuning: dict | None = None):
        lib = L.load()
        t = dict(tuning or {})
        if slots:
            t["slots"] = slots
        p = make_params(L.PPR, L.LOCAL_GD, prec, 1, 0.0, tau, tuning=t)
        h = ctypes.c_void_p()
        st = lib.gde_server_start(graph.ctx.ptr, graph.ptr, ctypes.byref(p), int(ring_capacity),
                                  float(hbm_budget_bytes), float(idle_ms), ctypes.byref(h))
        L.check(graph.ctx.ptr, st, "gde_server_start")
        self.ptr = h.value
        self.graph = graph
        self.ctx = graph.ctx
        self._rows = {}  # ticket -> caller buffer (kept alive until the query finishes)

    def submit(self, kind: int, seed: int, eps: float, alpha: float = 0.0, x_out=None, out64: bool = False) -> int:
        t = ctypes.c_int64()
        st = L.load().gde_server_submit(self.ptr, int(kind), int(seed), float(eps), float(alpha), _ptr(x_out),
                                        int(out64), ctypes.byref(t))
        L.check(self.ctx.ptr, st, "gde_server_submit")
        if x_out is not None:
            self._rows[t.value] = x_out
        return int(t.value)

    def poll(self, ticket: int):
        done, oper, rounds, dms = ctypes.c_int(), ctypes.c_double(), ctypes.c_int32(), ctypes.c_double()
        st = L.load().gde_server_poll(self.ptr, int(ticket), ctypes.byref(done), ctypes.byref(oper),
                                      ctypes.byref(rounds), ctypes.byref(dms))
        L.check(self.ctx.ptr, st, "gde_server_poll")
        if not done.value:
            return None
        self._rows.pop(int(ticket), None)
        return {"oper": oper.value, "rounds": rounds.value, "device_ms": dms.value}

    def poll_many(self, tickets: np.ndarray) -> dict:
        """Vector poll: dict(done[k] int32, oper[k], rounds[k], device_ms[k]) for int64 tickets."""
        tickets = np.ascontiguousarray(tickets, dtype=np.int64)
        k = tickets.shape[0]
        out = {"done": np.zeros(k, np.int32), "oper": np.zeros(k), "rounds": np.zeros(k, np.int32),
               "device_ms": np.zeros(k)}
        st = L.load().gde_server_poll_many(self.ptr, _ptr(tickets), k, _ptr(out["done"]), _ptr(out["oper"]),
                                           _ptr(out["rounds"]), _ptr(out["device_ms"]))
        L.check(self.ctx.ptr, st, "gde_server_poll_many")
        return out

    def info(self) -> dict:
        s, la, km, sub = ctypes.c_int(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_int64()
        st = L.load().gde_server_info(self.ptr, ctypes.byref(s), ctypes.byref(la), ctypes.byref(km), ctypes.byref(sub))
        return {"slots": s.value, "launches": la.value, "kernel_ms": km.value, "submitted": sub.value, "status": st}

    def stop(self, drain: bool = True) -> int:
        """End the server; returns the number of queries abandoned (0 with drain)."""
        if self.ptr is None:
            return 0
        lost = ctypes.c_int64()
        st = L.load().gde_server_stop(self.ptr, int(drain), ctypes.byref(lost))
        self.ptr = None
        self._rows.clear()
        L.check(self.ctx.ptr, st, "gde_server_stop")
        return int(lost.value)

    def __del__(self):
        if getattr(self, "ptr", None) is not None:
            try:
                self.stop(drain=False)
            except Exception:
                pass


def sor(graph: Graph, kind: int, seeds, eps, *, omega: float, local: bool = True, alpha: float = 0.0,
        prec: str = "fp64", out64: bool | None = None, want_x: bool = True, want_r: bool = True,
        device_out: bool = False, max_sweeps: int = 0) -> dict:
    """Multicolour LocalSOR / global SOR (ppr_sor / katz_sor order on the GPU); dict(x, r, oper, sweeps, stats)."""
    lib = L.load()
    seeds = np.ascontiguousarray(np.atleast_1d(seeds), dtype=np.int32)
    nq = seeds.shape[0]
    eps = np.ascontiguousarray(np.broadcast_to(np.asarray(eps, dtype=np.float64), (nq,)))
    if out64 is None:
        out64 = prec == "fp64"
    n = graph.n
    x_out = _alloc((nq, n), out64, device_out, graph) if want_x else None
    r_out = _alloc((nq, n), out64, device_out, graph) if want_r else None
    oper = np.zeros(nq, dtype=np.float64)
    sweeps = np.zeros(nq, dtype=np.int32)
    p = make_params(kind, L.LOCAL_GD, prec, 1, alpha, omega=omega, max_rounds=max_sweeps)
    st = L.Stats()
    status = lib.gde_sor(graph.ctx.ptr, graph.ptr, ctypes.byref(p), nq, _ptr(seeds), _ptr(eps), int(local),
                         _ptr(x_out), _ptr(r_out), int(out64), L.MEM_DEVICE if device_out else L.MEM_HOST, n,
                         _ptr(oper), _ptr(sweeps), ctypes.byref(st))
    L.check(graph.ctx.ptr, status, "gde_sor")
    return {"x": x_out, "r": r_out, "oper": oper, "sweeps": sweeps, "stats": st.as_dict()}


def graph_colors(graph: Graph) -> np.ndarray:
    """The proper colouring gde_sor uses, per caller node id."""
    lib = L.load()
    out = np.zeros(graph.n, dtype=np.int32)
    nc = ctypes.c_int32()
    L.check(graph.ctx.ptr, lib.gde_graph_colors(graph.ptr, _ptr(out), ctypes.byref(nc)), "gde_graph_colors")
    return out


def katz_spectral_bounds(graph: Graph, alpha: float, max_iter: int = 400, tol: float = 1e-10) -> dict:
    """lambda_max / lambda_min of the adjacency (GPU Lanczos) and the Katz Chebyshev bounds l_max, mu_min."""
    lib = L.load()
    out = [ctypes.c_double() for _ in range(4)]
    st = lib.gde_katz_spectral_bounds(graph.ctx.ptr, graph.ptr, float(alpha), int(max_iter), float(tol),
                                      *[ctypes.byref(o) for o in out])
    L.check(graph.ctx.ptr, st, "gde_katz_spectral_bounds")
    return {"lam_max": out[0].value, "lam_min": out[1].value, "l_max": out[2].value, "mu_min": out[3].value}


def _alloc(shape, out64: bool, device: bool, graph: Graph):
    if device:
        import torch
        return torch.empty(shape, dtype=torch.float64 if out64 else torch.float32, device=f"cuda:{graph.ctx.device}")
    return np.empty(shape, dtype=np.float64 if out64 else np.float32)


def ctx_stream(ctx: Context | None = None) -> int:
    """The library's CUDA stream handle (for torch.cuda.ExternalStream / events)."""
    c = ctx or Context.get(0)
    return int(L.load().gde_ctx_stream(c.ptr) or 0)


def set_wait_limit(polls: int, ctx: Context | None = None) -> None:
    """Polls before a bounded device wait gives up with GDE_EHANG (0: the library's defaults)."""
    c = ctx or Context.get(0)
    L.check(c.ptr, L.load().gde_ctx_set_wait_limit(c.ptr, int(polls)), "gde_ctx_set_wait_limit")


def trace(iters: int, ctx: Context | None = None) -> None:
    """Record per-block phase stamps for the first ``iters`` iterations of later push launches (0 = off)."""
    c = ctx or Context.get(0)
    L.check(c.ptr, L.load().gde_ctx_trace(c.ptr, int(iters)), "gde_ctx_trace")


def trace_read(ctx: Context | None = None) -> np.ndarray:
    """Stamps (ns) of the last push launch as [iters, grid, points]; 0 = point not reached."""
    c = ctx or Context.get(0)
    lib = L.load()
    it, gr, pt = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    L.check(c.ptr, lib.gde_ctx_trace_read(c.ptr, None, 0, ctypes.byref(it), ctypes.byref(gr), ctypes.byref(pt)),
            "gde_ctx_trace_read")
    out = np.zeros((it.value, gr.value, pt.value), dtype=np.uint64)
    if out.size:
        L.check(c.ptr, lib.gde_ctx_trace_read(c.ptr, _ptr(out), out.size, None, None, None), "gde_ctx_trace_read")
    return out


def feature_push(graph: Graph, kind: int, P, R, eps: float, *, alpha: float, beta: float = 0.0, prec: str = "fp64",
                 cand=None, tile_w: int = 0, max_rounds: int = 0, tuning: dict | None = None,
                 omega: float = 1.0) -> dict:
    """Multi-column push on device matrices P, R ([n, F] torch tensors), in place.

    ``omega != 1``: relaxed push in multicolour SOR order (instantGNNSorPush for GDE_IGN,
    update_ppr's push for GDE_UPPR).
    """
    lib = L.load()
    F = int(P.shape[1])
    ld = int(P.stride(0))
    assert R.stride(0) == ld and P.is_cuda and R.is_cuda
    p = make_params(kind, L.LOCAL_GD, prec, tile_w, alpha=alpha, beta=beta, omega=omega, max_rounds=max_rounds,
                    tuning=tuning)
    oper = np.zeros(F, dtype=np.float64)
    st = L.Stats()
    c = None if cand is None else np.ascontiguousarray(cand, dtype=np.int32)
    status = lib.gde_feature_push(graph.ctx.ptr, graph.ptr, ctypes.byref(p), F, _ptr(P), _ptr(R), ld, eps, _ptr(c),
                                  0 if c is None else c.shape[0], _ptr(oper), ctypes.byref(st))
    L.check(graph.ctx.ptr, status, "gde_feature_push")
    return {"oper": oper, "stats": st.as_dict()}


def feature_update(graph: Graph, kind: int, h_indices: np.ndarray, h_degree: np.ndarray, us, vs, only_insert: bool,
                   P, R, X, eps: float, *, alpha: float, beta: float = 0.0, prec: str = "fp64", tile_w: int = 0,
                   max_rounds: int = 0, omega: float = 1.0) -> dict:
    """Edge batch + repair + push (device P, R, X; host graph arrays mutated in place)."""
    lib = L.load()
    assert h_indices.dtype == np.int32 and h_degree.dtype == np.int64
    assert h_indices.flags.c_contiguous and h_degree.flags.c_contiguous
    us = np.ascontiguousarray(us, dtype=np.int32)
    vs = np.ascontiguousarray(vs, dtype=np.int32)
    F = int(P.shape[1])
    ld = int(P.stride(0))
    p = make_params(kind, L.LOCAL_GD, prec, tile_w, alpha=alpha, beta=beta, omega=omega, max_rounds=max_rounds)
    oper = np.zeros(F, dtype=np.float64)
    st = L.Stats()
    status = lib.gde_feature_update(graph.ctx.ptr, graph.ptr, _ptr(h_indices), _ptr(h_degree), _ptr(us), _ptr(vs),
                                    us.shape[0], int(only_insert), ctypes.byref(p), F, _ptr(P), _ptr(R), _ptr(X), ld,
                                    eps, _ptr(oper), ctypes.byref(st))
    L.check(graph.ctx.ptr, status, "gde_feature_update")
    return {"oper": oper, "stats": st.as_dict()}


def graph_update(graph: Graph, h_indices: np.ndarray, h_degree: np.ndarray, us, vs, only_insert: bool) -> dict:
    """The edge batch alone on the padded CSR (updetaGraph semantics); host arrays mutated in place.

    Returns dict(outcome, stats): outcome[i] = 0 no change, 1 inserted, 2 deleted.
    """
    lib = L.load()
    assert h_indices.dtype == np.int32 and h_degree.dtype == np.int64
    assert h_indices.flags.c_contiguous and h_degree.flags.c_contiguous
    us = np.ascontiguousarray(us, dtype=np.int32)
    vs = np.ascontiguousarray(vs, dtype=np.int32)
    outcome = np.zeros(us.shape[0], dtype=np.uint8)
    st = L.Stats()
    status = lib.gde_graph_update(graph.ctx.ptr, graph.ptr, _ptr(h_indices), _ptr(h_degree), _ptr(us), _ptr(vs),
                                  us.shape[0], int(only_insert), _ptr(outcome), ctypes.byref(st))
    L.check(graph.ctx.ptr, status, "gde_graph_update")
    return {"outcome": outcome, "stats": st.as_dict()}


def feature_repair(graph: Graph, kind: int, P, R, X, keys, old_degree, nbr_off, nbr, *, alpha: float,
                   beta: float = 0.0, prec: str = "fp64") -> None:
    """Repair device matrices P, R ([n, F]) at the keys after an edge batch (instantGNNUpdateBatch / update_ppr)."""
    lib = L.load()
    F = int(P.shape[1])
    ld = int(P.stride(0))
    keys = np.ascontiguousarray(keys, dtype=np.int32)
    old_degree = np.ascontiguousarray(old_degree, dtype=np.int64)
    nbr_off = np.ascontiguousarray(nbr_off, dtype=np.int64)
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    p = make_params(kind, L.LOCAL_GD, prec, 0, alpha=alpha, beta=beta)
    status = lib.gde_feature_repair(graph.ctx.ptr, graph.ptr, ctypes.byref(p), F, _ptr(P), _ptr(R), _ptr(X), ld,
                                    keys.shape[0], _ptr(keys), _ptr(old_degree), _ptr(nbr_off),
                                    _ptr(nbr) if nbr.size else None)
    L.check(graph.ctx.ptr, status, "gde_feature_repair")


def repad(graph: Graph, min_slack: int) -> tuple[np.ndarray, np.ndarray]:
    """Re-lay a padded graph with at least ``min_slack`` free slots per row, on the device.

    Returns the new host ``(indptr, indices)``; the caller's degree array stays valid.
    """
    lib = L.load()
    cap = ctypes.c_int64()
    L.check(graph.ctx.ptr, lib.gde_graph_repad(graph.ctx.ptr, graph.ptr, int(min_slack), None, None,
                                                ctypes.byref(cap)), "gde_graph_repad")
    indptr = np.empty(graph.n + 1, dtype=np.int64)
    indices = np.empty(max(cap.value, 1), dtype=np.int32)[:cap.value]
    L.check(graph.ctx.ptr, lib.gde_graph_repad(graph.ctx.ptr, graph.ptr, int(min_slack), _ptr(indptr), _ptr(indices),
                                                ctypes.byref(cap)), "gde_graph_repad")
    return indptr, indices


def plain_ppr_local(graph: Graph, seed: int, alpha: float, eps: float, x_out=None, r_out=None):
    """The plain single-query baseline (structure of ppr_gd_local_gpu)."""
    lib = L.load()
    oper = ctypes.c_double()
    rounds = ctypes.c_int32()
    status = lib.gde_plain_ppr_local(graph.ctx.ptr, graph.ptr, int(seed), alpha, eps, _ptr(x_out), _ptr(r_out),
                                     ctypes.byref(oper), ctypes.byref(rounds))
    L.check(graph.ctx.ptr, status, "gde_plain_ppr_local")
    return oper.value, rounds.value


def probe_random_atomics(n_floats: int, with_return: bool = True, ctx: Context | None = None) -> float:
    """Uniformly random FP32 atomic adds over ``n_floats`` entries, in G atomics/s (the push's ceiling)."""
    c = ctx or Context.get(0)
    out = ctypes.c_double()
    L.check(c.ptr, L.load().gde_probe_random_atomics(c.ptr, int(n_floats), int(with_return), ctypes.byref(out)),
            "gde_probe_random_atomics")
    return float(out.value)


def hk_estimate_n(tau: float, eps: float) -> int:
    return int(L.load().gde_hk_estimate_n(tau, eps))


def sync(ctx: Context | None = None) -> None:
    c = ctx or Context.get(0)
    L.check(c.ptr, L.load().gde_ctx_sync(c.ptr), "gde_ctx_sync")
