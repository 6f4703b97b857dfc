#!/usr/bin/env python
"""Benchmark: PPR queries/s and p50/p99 latency at eps=1e-7, FP32 batched local push, one GB300.

Workload (the configuration the headline metric is quoted on): the
wiki-talk-shaped Chung-Lu graph (n = 2,364,073, 9,355,158 CSR entries,
degree exponent ~2, max degree ~62k), personalized PageRank local GD with
alpha = 0.1, eps = 1e-7, seeds drawn uniformly from nodes with degree >= 1.
One step = one batch of --batch queries solved to the reference's stopping
rule by the GPU engine (FP32 residuals, Kahan FP32 solution, FP64 threshold
tests), results left in HBM.  `e2e` repeats the step through the public C
ABI with host seeds/eps and the solution rows copied back to pinned host
memory inside the timed region.

Reported beside it: the plain single-query GPU baseline (the structure of
the reference's ppr_gd_local_gpu on this GPU, the denominator of the
speed-up), and the timed CPU baseline (the C port of the reference's
ppr_gd local, FP64, all host cores, a bounded sample of queries).

--impl reference times the reference's CPU implementation of the path (the
C port in oracle/, the reference itself being numba Python that is not
installed on the GPU machine) on the same workload and prints the same line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "faster-local-solver-for-gdes_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "PPR queries/s + p50/p99 ms at ε=1e-7, served FP32 vs plain local push, 1 GB300"
ALPHA = 0.1
EPS = 1e-7
WORKLOAD = "ppr_local_gd_fp32_batched_chung_lu_2.36M"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=1024, help="queries per step")
    ap.add_argument("--tile-w", type=int, default=1, help="1 = served slots (continuous batching)")
    ap.add_argument("--slots", type=int, default=64,
                    help="concurrent queries of the served engine (each slot advances behind its own block "
                         "group's barrier; --tuning groups=G to share groups)")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--plain-queries", type=int, default=32)
    ap.add_argument("--cpu-queries", type=int, default=0, help="CPU-baseline sample (0 = 2 per host thread)")
    ap.add_argument("--no-baselines", action="store_true")
    ap.add_argument("--tuning", default="", help="k=v,... engine tuning overrides")
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c2arms", "c3", "c4", "c5"],
                    help="c1: FP64 local GD, 50 seeds on the 100k graph, checked against a global solve; "
                         "c2arms: local GD and local Chebyshev in FP64 and FP32 on the 2.36M graph; "
                         "c2: served PPR on the 2.36M graph (the headline); c3: 1,024 seeds per launch with "
                         "per-seed eps on the 100k graph; c4: served PPR/Katz/heat-kernel mix with Poisson "
                         "arrivals on R-MAT scale 22; c5: InstantGNN 128-column snapshot updates")
    ap.add_argument("--edit", default="insert", choices=["insert", "mixed"],
                    help="c5: insert-only snapshots, or a sliding window that also deletes the previous snapshot's "
                         "edges (updetaGraph with onlyinsert = False)")
    ap.add_argument("--mlp", action="store_true",
                    help="c5: train the MLP classifier on the device-resident features after the initial push and "
                         "after the last snapshot (outside the timed region)")
    ap.add_argument("--online", action="store_true",
                    help="c4: submit the queries in real time to the online server (gde_server_*) instead of "
                         "handing the whole arrival schedule to one served launch")
    ap.add_argument("--max-p99-ms", type=float, default=None,
                    help="c3: the autotuner keeps the fastest configuration whose p99 query latency is within this")
    ap.add_argument("--rates", default="250,500,1000,2000,0",
                    help="c4: Poisson arrival rates in queries/s to sweep (0 = all queries at once)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            import tempfile
            self.fh = tempfile.NamedTemporaryFile("w+", prefix="gde_clocks_", suffix=".csv", delete=False)
            self.path = self.fh.name
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self) -> dict:
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            lines = fh.readlines()
        os.unlink(self.path)
        for line in lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        if d.get("hbm_gbs"):
            return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic():
    """Per-launch DRAM traffic of the push kernel from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "push_kernel_traffic.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d
    return None


def algorithmic_bytes(stats: dict) -> float:
    """FP32: 4 B col_idx per union-frontier edge, 8 B residual RMW per (edge, column),
    32 B per active (node, column): row_ptr pair, r read/zero, x RMW, degree, frontier index."""
    return 4.0 * stats["union_vol"] + 8.0 * stats["col_vol"] + 32.0 * stats["col_nodes"]


def cpu_baseline(g, n_queries: int, eps: float):
    from oracle import oracle as O
    threads = O.threads()
    if n_queries <= 0:
        n_queries = 2 * threads
    from gde import graphs
    seeds = graphs.uniform_seeds(g, n_queries, seed=424242)
    deg = g.degree.astype(np.float64)
    t0 = time.perf_counter()
    O.ppr_gd_many(g.n, g.indptr, g.indices, deg, seeds, ALPHA, eps, local=True, nthreads=threads)
    dt = time.perf_counter() - t0
    return n_queries / dt, threads, n_queries, dt


def accuracy_vs_oracle(G, g, tuning, n_queries: int = 8):
    """FP32 served results against the FP64 oracle on a few of the workload's queries (outside any timing)."""
    from gde import _lib as L
    from gde import api, graphs
    from oracle import oracle as O
    seeds = graphs.uniform_seeds(g, n_queries, seed=515151)
    deg = g.degree.astype(np.float64)
    oper_o, x_o = O.ppr_gd_many(g.n, g.indptr, g.indices, deg, seeds, ALPHA, EPS, local=True, keep_x=True)
    res = api.solve(G, L.PPR, L.LOCAL_GD, seeds, EPS, prec="fp32", alpha=ALPHA, tile_w=1, want_r=False,
                    tuning=tuning)
    rel = [float(np.abs(res["x"][i] - x_o[i]).sum() / np.abs(x_o[i]).sum()) for i in range(n_queries)]
    absl1 = [float(np.abs(res["x"][i] - x_o[i]).sum()) for i in range(n_queries)]
    od = [abs(float(res["oper"][i]) - float(oper_o[i])) / float(oper_o[i]) for i in range(n_queries)]
    out = {"vs": "FP64 oracle (C port of ppr_gd local)", "queries": n_queries, "eps": EPS,
           "l1_mean": float(np.mean(absl1)), "l1_max": float(np.max(absl1)),
           "rel_l1_mean": float(np.mean(rel)), "rel_l1_max": float(np.max(rel)),
           "oper_rel_diff_max": float(np.max(od))}
    out["truth"] = accuracy_vs_truth(G, g, seeds[:2], x_o[:2], tuning)
    return out


def accuracy_vs_truth(G, g, seeds, x_oracle, tuning):
    """FP32 served results against the PPR vector itself: an FP64 global solve (Jacobi on the
    device in torch, to ||r||_1 < 1e-14), with the oracle's own distance to it for scale, and the
    largest D^-1 residual left by the served solve (its stopping rule is max r_u / d_u < eps alpha)."""
    import torch
    from gde import _lib as L
    from gde import api
    dev = f"cuda:{G.ctx.device}"
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")  # torch flags its sparse CSR support as beta
        A = torch.sparse_csr_tensor(torch.from_numpy(g.indptr.astype(np.int64)),
                                    torch.from_numpy(g.indices.astype(np.int64)),
                                    torch.ones(g.indices.shape[0], dtype=torch.float64), size=(g.n, g.n)).to(dev)
    dinv = torch.from_numpy(1.0 / g.degree.astype(np.float64)).to(dev)
    res = api.solve(G, L.PPR, L.LOCAL_GD, seeds, EPS, prec="fp32", alpha=ALPHA, tile_w=1, want_r=True, tuning=tuning)
    rows = []
    for i, s in enumerate(seeds):
        r = torch.zeros(g.n, dtype=torch.float64, device=dev)
        r[int(s)] = ALPHA
        x = torch.zeros_like(r)
        for _ in range(2000):  # x = alpha (I - (1-alpha) A D^-1)^-1 e_s
            x += r
            r = (1.0 - ALPHA) * (A @ (r * dinv).unsqueeze(1)).squeeze(1)
            if float(r.abs().sum()) < 1e-14:
                break
        truth = (x + r).cpu().numpy()
        xg = res["x"][i].astype(np.float64)
        rg = res["r"][i].astype(np.float64)
        rows.append({"l1": float(np.abs(xg - truth).sum()), "oracle_l1": float(np.abs(x_oracle[i] - truth).sum()),
                     "max_r_over_d": float(np.max(np.abs(rg) / g.degree))})
    return {"vs": "FP64 global solve to 1e-14 (torch, on the device)", "queries": len(rows),
            "l1_max": max(r["l1"] for r in rows), "oracle_l1_max": max(r["oracle_l1"] for r in rows),
            "max_r_over_d": max(r["max_r_over_d"] for r in rows), "stop_rule": EPS * ALPHA}


def c2_config(g, Q, args, world):
    """The headline workload, named the same in both arms (the reference arm times a sample of it)."""
    return {"workload": WORKLOAD, "n": g.n, "nnz": g.nnz, "queries_per_step": Q, "alpha": ALPHA, "eps": EPS,
            "tile_w": args.tile_w, "slots": args.slots,
            "precision": "fp32 residual, kahan fp32 x, fp64 threshold",
            "l2": "512 MB buffer written between timed steps", "parallelism": f"replicas x{world}"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from gde import graphs
    from oracle import oracle as O
    O.build()
    g = graphs.chung_lu_wikitalk_shape()
    threads = O.threads()
    per_step = max(args.cpu_queries, threads)
    deg = g.degree.astype(np.float64)
    for w in range(args.warmup):
        O.ppr_gd_many(g.n, g.indptr, g.indices, deg, graphs.uniform_seeds(g, threads, seed=900 + w), ALPHA, EPS,
                      nthreads=threads)
    t_total = 0.0
    for s in range(args.steps):
        seeds = graphs.uniform_seeds(g, per_step, seed=1000 + s)
        t0 = time.perf_counter()
        O.ppr_gd_many(g.n, g.indptr, g.indices, deg, seeds, ALPHA, EPS, nthreads=threads)
        t_total += time.perf_counter() - t0
    qps = per_step * args.steps / t_total
    line = {
        "metric": METRIC, "value": qps, "unit": "queries/s", "impl": "reference", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": c2_config(g, args.batch, args, 1),
        "sample_queries_per_step": per_step,
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": f"{per_step} of the workload's queries per step (ppr_gd local FP64, the C port "
                                   f"of the reference), one per OpenMP thread"},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from gde import _lib as L
    from gde import api, graphs

    tuning = dict(parse_tuning(args.tuning), slots=args.slots)
    g = graphs.chung_lu_wikitalk_shape()
    ctx = api.Context.get(local)
    G = api.Graph(g.indptr, g.indices, ctx=ctx)
    Q = args.batch
    stream = torch.cuda.ExternalStream(api.ctx_stream(ctx), device=f"cuda:{local}")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")  # > L2 (129 MB)
    x_dev = torch.empty((Q, g.n), dtype=torch.float32, device=f"cuda:{local}")

    def step(seed_base, x_out=None, device_out=True):
        seeds = graphs.uniform_seeds(g, Q, seed=seed_base)
        return api.solve(G, L.PPR, L.LOCAL_GD, seeds, EPS, prec="fp32", alpha=ALPHA, tile_w=args.tile_w,
                         want_r=False, x_out=x_out if x_out is not None else x_dev, device_out=device_out,
                         tuning=tuning)

    for w in range(args.warmup):
        step(10_000 * rank + w)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()

    times = []
    lat = []
    kms = []
    ph = {"check": [], "prep": [], "scatter": []}
    agg = {"union_vol": 0.0, "col_vol": 0.0, "col_nodes": 0, "union_nodes": 0, "rounds": 0}
    opers = []
    launches = 0
    with ClockSampler(local) as clk:
        for s in range(args.steps):
            flush.zero_()  # L2 flush between timed steps
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            res = step(20_000 * rank + 100 + s)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            st = res["stats"]
            kms.append(st["kernel_ms"])
            for k in ph:
                ph[k].append(st[k + "_ms"])
            for k in agg:
                agg[k] += st[k]
            lat.extend(res["latency_ms"].tolist())
            opers.extend(res["oper"].tolist())
            launches += max(1, int(np.ceil(st["tiles"] / 4096)))
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    total_ms = float(sum(times))
    if world > 1:
        t = torch.tensor([total_ms], device=f"cuda:{local}", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = Q * args.steps * world / (total_ms / 1e3)

    # ---- end to end through the C ABI with host buffers ----
    x_host = torch.empty((Q, g.n), dtype=torch.float32).pin_memory()
    e2e_ms = []
    if args.e2e_steps:
        step(30_000 * rank + 999, x_out=x_host, device_out=False)  # untimed: first use of the host rows
    for s in range(args.e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step(30_000 * rank + s, x_out=x_host, device_out=False)
        e1.record(stream)
        e1.synchronize()
        e2e_ms.append(e0.elapsed_time(e1))
    e2e_total = float(sum(e2e_ms))
    if world > 1 and e2e_ms:
        t = torch.tensor([e2e_total], device=f"cuda:{local}", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)  # the slowest replica
        e2e_total = float(t.item())
    e2e_value = Q * max(1, args.e2e_steps) * world / (e2e_total / 1e3) if e2e_ms else None

    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return

    peak, peak_kind = measured_peak()
    kernel_ms_total = float(sum(kms))
    bytes_total = algorithmic_bytes(agg)
    achieved = bytes_total / (kernel_ms_total / 1e3) / 1e9
    traffic = committed_traffic()
    per_launch_bytes = bytes_total / launches
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": peak_kind,
            # the small capture's DRAM bytes per edge operation, scaled to this
            # launch's operations (traffic grows with the pushes)
            "traffic": (traffic["dram_bytes_per_oper"] * float(np.sum(opers)) / launches
                        if traffic and opers else None),
            "algorithmic_bytes_per_launch": per_launch_bytes, "kernel": "push_kernel<float,%d>" % args.tile_w,
            "kernel_ms_per_launch": kernel_ms_total / launches}
    lat_sorted = np.sort(np.asarray(lat))
    out = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": c2_config(g, Q, args, world),
        "p50_ms": float(np.percentile(lat_sorted, 50)) if lat else None,
        "p99_ms": float(np.percentile(lat_sorted, 99)) if lat else None,
        "mean_oper": float(np.mean(opers)) if opers else None,
        "rounds_total": agg["rounds"],
        "phase_ms": {k: float(sum(ph[k])) / args.steps for k in ph},
        # per served step: the push launch, the slot seeding and the solution read-out
        "gpu_launches": int(launches + args.steps * 2),
        "roofline": roof,
        "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": Q * (4 + 8),
                "d2h_bytes_per_step": Q * g.n * 4 + Q * (8 + 4 + 4)},
    }
    out["clocks"] = clk.summary()
    # the push's own ceiling: uniformly random FP32 atomics (with return) over
    # an array the size of the slots' residual slabs, against the SCATTER
    # phase's edge-push rate (its time includes the phase's barrier wait)
    foot = int(res["stats"]["tiles"]) * args.tile_w * g.n
    probe = api.probe_random_atomics(foot, True, ctx)
    scat_rate = agg["col_vol"] / (sum(ph["scatter"]) / 1e3) / 1e9
    out["random_access"] = {"scatter_atomics_gps": scat_rate, "probe_atomics_gps": probe,
                            "frac": scat_rate / probe, "footprint_mb": foot * 4 / 1e6}
    if not args.no_baselines:
        # plain single-query GPU baseline (the x20 denominator)
        xs = torch.zeros(g.n, dtype=torch.float32, device=f"cuda:{local}")
        seeds = graphs.uniform_seeds(g, args.plain_queries + 1, seed=777)
        api.plain_ppr_local(G, int(seeds[0]), ALPHA, EPS, x_out=xs)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s in seeds[1:]:
            api.plain_ppr_local(G, int(s), ALPHA, EPS, x_out=xs)
        torch.cuda.synchronize()
        plain_qps = args.plain_queries / (time.perf_counter() - t0)
        out["plain_gpu"] = {"value": plain_qps, "unit": "queries/s", "sample": f"{args.plain_queries} queries",
                            "speedup": value / plain_qps}
        qps, threads, nq, dt = cpu_baseline(g, args.cpu_queries, EPS)
        out["cpu_baseline"] = {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                               "sample": f"{nq} queries (ppr_gd local FP64, one per OpenMP thread), {dt:.1f} s"}
        out["accuracy"] = accuracy_vs_oracle(G, g, tuning)
    print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.barrier()


def _timed_steps(stream, flush, steps, fn, warm=0):
    """CUDA-event time of each step on the library stream, L2 flushed before each (after ``warm`` untimed steps)."""
    import torch
    times = []
    outs = []
    for s in range(warm):
        fn(10_000 + s)
    for s in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        outs.append(fn(s))
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    return times, outs


def run_c3(args):
    """Batched PPR: 1,024 seeds per launch on the 100k-node graph, eps log-uniform in [1e-8, 1e-5]."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    from gde import _lib as L
    from gde import api, graphs, tune
    g = graphs.chung_lu_100k()
    ctx = api.Context.get(local)
    G = api.Graph(g.indptr, g.indices, ctx=ctx)
    Q = 1024

    def batch(k):
        rng = np.random.default_rng(2 + 1000 * rank + k)
        return graphs.uniform_seeds(g, Q, seed=2 + 1000 * rank + k), np.exp(rng.uniform(np.log(1e-8), np.log(1e-5), Q))

    s0, e0 = batch(0)
    # the tuner times each configuration on the step's own queries: a smaller sample favours node x seed
    # tiles, whose residual slabs fit in the L2 at a quarter of the tiles but not at the step's size
    best = tune.autotune(G, L.PPR, s0, e0, prec="fp32", alpha=ALPHA, max_p99_ms=args.max_p99_ms)
    best = dict(best, tuning=dict(best["tuning"], **parse_tuning(args.tuning)))  # --tuning overrides
    stream = torch.cuda.ExternalStream(api.ctx_stream(ctx), device=f"cuda:{local}")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    x_dev = torch.empty((Q, g.n), dtype=torch.float32, device=f"cuda:{local}")

    def step(k, x_out=None, device_out=True):
        sd, ep = batch(k)
        return api.solve(G, L.PPR, L.LOCAL_GD, sd, ep, prec="fp32", alpha=ALPHA, tile_w=best["tile_w"],
                         tuning=best["tuning"], want_r=False, x_out=x_dev if x_out is None else x_out,
                         device_out=device_out)

    for w in range(args.warmup):
        step(10 + w)
    with ClockSampler(local) as clk:
        times, outs = _timed_steps(stream, flush, args.steps, lambda k: step(100 + k))
    total_ms = sum(times)
    value = Q * args.steps * world / (total_ms / 1e3)
    agg = {k: sum(o["stats"][k] for o in outs) for k in ("union_vol", "col_vol", "col_nodes", "kernel_ms")}
    achieved = algorithmic_bytes(agg) / (agg["kernel_ms"] / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    lat = np.concatenate([o["latency_ms"] for o in outs])
    x_host = torch.empty((Q, g.n), dtype=torch.float32).pin_memory()
    e2e, _ = _timed_steps(stream, flush, max(1, args.e2e_steps), lambda k: step(200 + k, x_host, False), warm=1)
    out = {
        "metric": "batched PPR queries/s, 1,024 seeds per launch, eps log-uniform [1e-8, 1e-5], FP32",
        "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "ppr_local_gd_fp32_batched_1024_chung_lu_100k", "n": g.n, "nnz": g.nnz,
                   "queries_per_step": Q, "alpha": ALPHA, "eps": "log-uniform [1e-8, 1e-5]",
                   "autotuned": {"tile_w": best["tile_w"], "tuning": best["tuning"],
                                 "max_p99_ms": args.max_p99_ms},
                   "l2": "512 MB buffer written between timed steps"},
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": None},
        "e2e": {"value": Q * len(e2e) * world / (sum(e2e) / 1e3), "unit": "queries/s",
                "h2d_bytes_per_step": Q * 12, "d2h_bytes_per_step": Q * g.n * 4},
        "gpu_launches": args.steps, "clocks": clk.summary(),
        "autotune_table": best["table"],
    }
    if not args.no_baselines and rank == 0:
        from oracle import oracle as O
        threads = O.threads()
        # the last timed step's rows (still in x_dev) against the FP64 oracle: 64 of its 1,024 queries
        sd, ep = batch(100 + args.steps - 1)
        pick = np.arange(0, Q, Q // 64)
        oo, xo = O.ppr_gd_many(g.n, g.indptr, g.indices, g.degree.astype(np.float64), sd[pick], ALPHA, ep[pick],
                               keep_x=True, nthreads=threads)
        xg = x_dev[torch.from_numpy(pick).to(x_dev.device)].double().cpu().numpy()
        l1 = np.abs(xg - xo).sum(1)
        od = np.abs(outs[-1]["oper"][pick] - oo) / np.maximum(oo, 1)
        out["accuracy"] = {"vs": "FP64 oracle (C port of ppr_gd local)", "queries": int(pick.size),
                           "l1_max": float(l1.max()), "l1_mean": float(l1.mean()),
                           "rel_l1_max": float((l1 / np.abs(xo).sum(1)).max()),
                           "oper_rel_diff_max": float(od.max()), "oper_abs_diff_max": float(
                               np.abs(outs[-1]["oper"][pick] - oo).max())}
        sd, ep = batch(300)
        nq = max(args.cpu_queries, 2 * threads)
        t0 = time.perf_counter()
        O.ppr_gd_many(g.n, g.indptr, g.indices, g.degree.astype(np.float64), sd[:nq], ALPHA, ep[:nq], nthreads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": nq / dt, "unit": "queries/s", "cores": threads, "kind": "port",
                               "sample": f"{nq} of the step's queries (ppr_gd local FP64), {dt:.1f} s"}
    if rank == 0:
        print(json.dumps(out), flush=True)


def mixed_oracle(g, kind, seed, eps, alpha, tau):
    """FP64 oracle row of one mixed query, as the reference returns it -> (x, oper)."""
    from gde import _lib as L
    from oracle import oracle as O
    deg = g.degree.astype(np.float64)
    if kind == L.PPR:
        x, _, o = O.ppr_gd(g.n, g.indptr, g.indices, deg, int(seed), alpha, eps, True)
    elif kind == L.KATZ:
        x, _, o = O.katz_gd(g.n, g.indptr, g.indices, deg, int(seed), alpha, eps, True)
    else:
        _, x, _, o = O.hk_sor_queue(g.n, g.indptr, g.indices, deg, int(seed), tau, eps, 1.0, True)
    return x, float(o)


def mixed_accuracy(g, rows, opers, kinds, seeds, eps, alphas, tau, per_kind: int = 3, eps_min: float = 1e-6):
    """FP32 rows of a mixed queue against the FP64 oracle, `per_kind` queries of each kind with eps >= eps_min
    (the oracle is sequential; smaller eps is what the GPU is for), in parallel on the host's threads."""
    from concurrent.futures import ThreadPoolExecutor
    from gde import _lib as L
    pick = []
    for k in (L.PPR, L.KATZ, L.HK):
        idx = np.flatnonzero((kinds == k) & (eps >= eps_min))[:per_kind]
        pick += [int(i) for i in idx]
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        orc = list(ex.map(lambda i: mixed_oracle(g, int(kinds[i]), seeds[i], float(eps[i]), float(alphas[i]), tau),
                          pick))
    per = {}
    for i, (xo, oo) in zip(pick, orc):
        x = np.asarray(rows[i], dtype=np.float64)
        name = {int(L.PPR): "ppr", int(L.KATZ): "katz", int(L.HK): "hk"}[int(kinds[i])]
        d = per.setdefault(name, {"queries": 0, "l1_max": 0.0, "rel_l1_max": 0.0, "oper_rel_diff_max": 0.0})
        d["queries"] += 1
        l1 = float(np.abs(x - xo).sum())
        d["l1_max"] = max(d["l1_max"], l1)
        d["rel_l1_max"] = max(d["rel_l1_max"], l1 / max(float(np.abs(xo).sum()), 1e-300))
        d["oper_rel_diff_max"] = max(d["oper_rel_diff_max"], abs(float(opers[i]) - oo) / max(oo, 1.0))
    return {"vs": "FP64 oracle (C ports of ppr_gd, katz_gd, hk_sor_queue local)", "eps_min": eps_min, "per_kind": per}


def mixed_cpu_baseline(g, kinds, seeds, eps, alphas, tau, budget_s: float = 15.0):
    """The oracle's C ports on the host's threads over the mix (eps as drawn), until about budget_s of work."""
    from concurrent.futures import ThreadPoolExecutor
    threads = os.cpu_count() or 1
    done = 0
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        while done < len(kinds) and time.perf_counter() - t0 < budget_s:
            k = min(threads, len(kinds) - done)
            list(ex.map(lambda i: mixed_oracle(g, int(kinds[i]), seeds[i], float(eps[i]), float(alphas[i]), tau),
                        range(done, done + k)))
            done += k
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"{done} queries of the mix (eps as drawn, FP64 C ports, one per thread), {dt:.1f} s"}


def parse_tuning(text):
    """``k=v,...`` engine tuning overrides (integers, or floats such as sparse_eps=1e-6)."""
    out = {}
    for kv in filter(None, text.split(",")):
        k, v = kv.split("=")
        out[k] = float(v) if any(c in v for c in ".eE") else int(v)
    return out


def run_c4(args):
    """Served mixed queries on R-MAT scale 22: 60% PPR, 25% Katz, 15% heat kernel, Poisson arrivals."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    from gde import _lib as L
    from gde import api, graphs
    t0 = time.perf_counter()
    g = graphs.rmat_scale22()
    gen_s = time.perf_counter() - t0
    ctx = api.Context.get(local)
    G = api.Graph(g.indptr, g.indices, ctx=ctx)
    dmax = float(g.degree.max())
    Q = args.batch
    tau, budget = 5.0, 120e9
    x_dev = torch.empty((Q, g.n), dtype=torch.float32, device=f"cuda:{local}")
    stream = torch.cuda.ExternalStream(api.ctx_stream(ctx), device=f"cuda:{local}")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def queries(k, rate):
        rng = np.random.default_rng(7 + 1000 * rank + k)
        kinds = rng.choice(np.array([L.PPR, L.KATZ, L.HK], np.int32), size=Q, p=[0.60, 0.25, 0.15])
        seeds = graphs.uniform_seeds(g, Q, seed=7 + 1000 * rank + k)
        eps = np.exp(rng.uniform(np.log(1e-8), np.log(1e-5), Q))
        # ppr_gd's precondition eps * degree[s] <= 1 (ppr_solver.py:213) for hub seeds
        eps = np.where(kinds == L.PPR, np.minimum(eps, 1.0 / g.degree[seeds]), eps)
        alphas = np.where(kinds == L.KATZ, 0.5 / dmax, ALPHA)
        arr = None if rate <= 0 else np.cumsum(rng.exponential(1e3 / rate, Q))
        return kinds, seeds, eps, alphas, arr

    config = {"workload": "served_mix_ppr_katz_hk_fp32_rmat22", "n": g.n, "nnz": g.nnz, "queries_per_step": Q,
              "ppr_alpha": ALPHA, "katz_alpha": "0.5 / d_max", "hk_tau": tau, "eps": "log-uniform [1e-8, 1e-5]",
              "hbm_budget_bytes": budget, "requested_slots": args.slots, "graph_generation_s": gen_s}
    tuning = parse_tuning(args.tuning)
    if tuning:
        config["tuning"] = tuning
    if args.online:
        run_c4_online(args, g, G, x_dev, queries, config, tau, budget)
        return

    def step(k, rate, x_out=None, device_out=True):
        kinds, seeds, eps, alphas, arr = queries(k, rate)
        return api.serve_mixed(G, kinds, seeds, eps, alphas=alphas, tau=tau, arrival_ms=arr, hbm_budget_bytes=budget,
                               prec="fp32", x_out=x_dev if x_out is None else x_out, device_out=device_out,
                               slots=args.slots, tuning=tuning)

    for w in range(args.warmup):
        step(10 + w, 0)
    rows = []
    sat = None
    with ClockSampler(local) as clk:
        for rate in [float(r) for r in args.rates.split(",")]:
            times, outs = _timed_steps(stream, flush, args.steps, lambda k: step(100 + k, rate))
            lat = np.concatenate([o["latency_ms"] for o in outs])
            rows.append({"rate_qps": rate if rate > 0 else None, "queries_per_s": Q * len(times) / (sum(times) / 1e3),
                         "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                         "slots": int(outs[0]["stats"]["tiles"]), "ms_per_step": sum(times) / len(times),
                         "table_queries": int(sum(o["stats"]["sparse_queries"] for o in outs)),
                         "table_overflows": int(sum(o["stats"]["sparse_overflows"] for o in outs))})
            if rate <= 0:
                sat = (times, outs, 100 + len(times) - 1)
    best = max(rows, key=lambda r: r["queries_per_s"])
    out = {
        "metric": "served mixed queries/s + p50/p99 ms (60% PPR, 25% Katz, 15% heat kernel), R-MAT scale 22",
        "value": best["queries_per_s"], "unit": "queries/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": best["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(config, l2="512 MB buffer written between timed steps"),
        "p50_ms": best["p50_ms"], "p99_ms": best["p99_ms"], "rate_sweep": rows,
        "gpu_launches": args.steps * len(rows), "clocks": clk.summary(),
    }
    if sat is not None:
        # roofline of the push kernel over the saturation steps (all queries arrive at once)
        times, outs, last = sat
        agg = {k: sum(o["stats"][k] for o in outs) for k in ("union_vol", "col_vol", "col_nodes", "kernel_ms")}
        achieved = algorithmic_bytes(agg) / (agg["kernel_ms"] / 1e3) / 1e9
        peak, peak_kind = measured_peak()
        out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                           "peak_kind": peak_kind, "traffic": None, "kernel": "push_kernel<float,1>",
                           "kernel_ms_per_launch": agg["kernel_ms"] / len(outs),
                           "algorithmic_bytes_per_launch": algorithmic_bytes(agg) / len(outs)}
        # e2e: the same saturation step into pinned host rows (host seeds, eps, kinds)
        x_host = torch.empty((Q, g.n), dtype=torch.float32).pin_memory()
        e2e, _ = _timed_steps(stream, flush, max(1, args.e2e_steps), lambda k: step(300 + k, 0, x_host, False), warm=1)
        out["e2e"] = {"value": Q * len(e2e) / (sum(e2e) / 1e3), "unit": "queries/s",
                      "h2d_bytes_per_step": Q * (4 + 4 + 8 + 8), "d2h_bytes_per_step": Q * g.n * 4}
        if not args.no_baselines:
            kinds, seeds, eps, alphas, _ = queries(last, 0)
            xr = x_dev.cpu().numpy()
            out["accuracy"] = mixed_accuracy(g, xr, outs[-1]["oper"], kinds, seeds, eps, alphas, tau)
            out["cpu_baseline"] = mixed_cpu_baseline(g, kinds, seeds, eps, alphas, tau)
    print(json.dumps(out), flush=True)


def run_c4_online(args, g, G, x_dev, queries, config, tau, budget):
    """The C4 mix through the online server: a host loop submits each query at its Poisson arrival time while
    the server's persistent launch runs, and watches the completion records.  Latency is measured on the host,
    from a query's scheduled arrival to the moment its completed record is seen; throughput is queries over the
    time from the first arrival to the last completion."""
    from gde import _lib as L
    from gde import api
    Q = args.batch
    srv = api.Server(G, prec="fp32", slots=args.slots, tau=tau, ring_capacity=max(4096, 2 * Q),
                     hbm_budget_bytes=budget, idle_ms=50.0)

    def run(k, rate):
        kinds, seeds, eps, alphas, arr = queries(k, rate)
        arr = np.zeros(Q) if arr is None else arr
        tickets = np.full(Q, -1, np.int64)
        fin = np.full(Q, np.nan)
        opers = np.zeros(Q)
        nxt = 0
        t0 = time.perf_counter()
        while True:
            now = (time.perf_counter() - t0) * 1e3
            while nxt < Q and arr[nxt] <= now:
                tickets[nxt] = srv.submit(int(kinds[nxt]), int(seeds[nxt]), float(eps[nxt]), float(alphas[nxt]),
                                          x_dev[nxt])
                nxt += 1
            idx = np.flatnonzero((tickets >= 0) & np.isnan(fin))
            if idx.size:
                r = srv.poll_many(tickets[idx])
                hit = r["done"] == 1
                if hit.any():
                    fin[idx[hit]] = (time.perf_counter() - t0) * 1e3
                    opers[idx[hit]] = r["oper"][hit]
            if nxt == Q and not np.isnan(fin).any():
                break
        lat = fin - arr
        span = (fin.max() - arr.min()) / 1e3
        return {"rate_qps": rate if rate > 0 else None, "queries_per_s": Q / span,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))}, \
            (kinds, seeds, eps, alphas, opers)

    for w in range(args.warmup):
        run(10 + w, 0)
    rows = []
    last = None
    with ClockSampler(G.ctx.device) as clk:
        for rate in [float(r) for r in args.rates.split(",")]:
            for k in range(args.steps):
                row, q = run(100 + k, rate)
                rows.append(row)
                if rate <= 0:
                    last = q
    info = srv.info()
    srv.stop()
    sat = [r for r in rows if r["rate_qps"] is None]
    best = max(sat or rows, key=lambda r: r["queries_per_s"])
    sweep = {}
    for r in rows:
        key = r["rate_qps"] or 0
        d = sweep.setdefault(key, {"rate_qps": r["rate_qps"], "queries_per_s": [], "p50_ms": [], "p99_ms": []})
        for f in ("queries_per_s", "p50_ms", "p99_ms"):
            d[f].append(r[f])
    sweep = [{k: (float(np.median(v)) if isinstance(v, list) else v) for k, v in d.items()} for d in sweep.values()]
    out = {
        "metric": "online served mixed queries/s + p50/p99 ms (60% PPR, 25% Katz, 15% heat kernel), R-MAT scale 22",
        "value": best["queries_per_s"], "unit": "queries/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * Q / best["queries_per_s"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(config, workload="online_served_mix_ppr_katz_hk_fp32_rmat22", submission="host loop, "
                       "real-time Poisson arrivals into the server's pinned ring", slots=info["slots"]),
        "p50_ms": best["p50_ms"], "p99_ms": best["p99_ms"], "rate_sweep": sweep,
        "server": info, "gpu_launches": int(info["launches"]), "clocks": clk.summary(),
        "latency": "host-observed: scheduled arrival to completion record seen",
    }
    if last is not None and not args.no_baselines:
        kinds, seeds, eps, alphas, opers = last
        out["accuracy"] = mixed_accuracy(g, x_dev.cpu().numpy(), opers, kinds, seeds, eps, alphas, tau)
    print(json.dumps(out), flush=True)


def run_c5(args):
    """InstantGNN dynamic propagation: 128 FP32 feature columns, 16 snapshots of 59,375 inserted edges."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    from gde import _lib as L
    from gde import api, graphs
    base = graphs.chung_lu_arxiv_shape()
    F, snaps, beta, eps = 128, 16, 0.5, 1e-7
    dyn = graphs.dynamic_padded(base, 950_000, snaps, seed=1)
    n = dyn.n
    rng = np.random.default_rng(3)
    X = rng.standard_normal((n, F)).astype(np.float32)
    dev = f"cuda:{local}"
    indices = dyn.indices.copy()
    degree = dyn.degree.copy()
    G = api.Graph(dyn.indptr, indices, row_len=degree, degree=degree.astype(np.float64), ctx=api.Context.get(local))
    Xd = torch.from_numpy(X).to(dev)
    Pd = torch.zeros_like(Xd)
    Rd = Xd.clone()
    stream = torch.cuda.ExternalStream(api.ctx_stream(G.ctx), device=dev)
    # --tuning tile_w=W: columns per tile (0 = the library's default)
    tw = int(dict(kv.split("=") for kv in filter(None, args.tuning.split(","))).get("tile_w", 0))
    t0 = time.perf_counter()
    api.feature_push(G, L.IGN, Pd, Rd, eps, alpha=ALPHA, beta=beta, prec="fp32", tile_w=tw)
    torch.cuda.synchronize()
    init_s = time.perf_counter() - t0
    mlp = {}
    if args.mlp:
        # 40 classes from a random linear map of the features (argmax), random 60/20/20 split;
        # the propagated matrix goes to torch on the device
        from gde import consumer
        labels = torch.from_numpy((X @ rng.standard_normal((F, 40))).argmax(1)).to(dev)
        split = consumer.random_split(n, dev, seed=4)
        mlp["initial"] = consumer.train_eval(Pd, labels, split)
    mixed = args.edit == "mixed"
    batches = []
    for s in range(snaps):
        us, vs = dyn.Us[s], dyn.Vs[s]
        if mixed and s > 0:
            # the previous snapshot's edges leave while this one's arrive, shuffled together
            perm = np.random.default_rng(100 + s).permutation(2 * us.shape[0])
            us = np.concatenate([dyn.Us[s - 1], us])[perm]
            vs = np.concatenate([dyn.Vs[s - 1], vs])[perm]
        batches.append((np.ascontiguousarray(us, dtype=np.int32), np.ascontiguousarray(vs, dtype=np.int32)))
    times, outs, snapP = [], [], []
    with ClockSampler(local) as clk:
        for s in range(snaps):
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            outs.append(api.feature_update(G, L.IGN, indices, degree, batches[s][0], batches[s][1], not mixed, Pd,
                                           Rd, Xd, eps, alpha=ALPHA, beta=beta, prec="fp32", tile_w=tw))
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            snapP.append(Pd[:, :C5_CHECK_COLS].double().cpu().numpy())  # after the timed region
    total_ms = sum(times)
    agg = {k: sum(o["stats"][k] for o in outs) for k in ("union_vol", "col_vol", "col_nodes", "kernel_ms")}
    achieved = algorithmic_bytes(agg) / (max(agg["kernel_ms"], 1e-9) / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    edits = f"{int(dyn.Us.shape[1]):,} inserted" + (" and as many deleted" if mixed else "")
    out = {
        "metric": f"InstantGNN snapshot updates/s (128 FP32 columns, {edits} edges per snapshot)",
        "value": snaps / (total_ms / 1e3), "unit": "snapshots/s", "n_gpus": 1, "steps": snaps, "warmup": 0,
        "ms_per_step": total_ms / snaps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "instantgnn_update_" + ("mixed_" if mixed else "") + "fp32_128col_chung_lu_169k",
                   "n": n, "features": F,
                   "snapshots": snaps, "edges_per_snapshot": int(dyn.Us.shape[1]), "alpha": ALPHA, "beta": beta,
                   "eps": eps, "initial_push_s": init_s, "tile_w": tw or "default"},
        "column_updates_per_s": snaps * F / (total_ms / 1e3),
        "push_kernel_ms_per_step": agg["kernel_ms"] / snaps,
        "phase_ms_per_step": {k: sum(o["stats"][k + "_ms"] for o in outs) / snaps for k in ("check", "prep", "scatter")},
        "edit_ms_per_step": sum(o["stats"]["edit_ms"] for o in outs) / snaps,
        "edit_paths": {p: sum(1 for o in outs if o["stats"]["edit_path"] == i)
                       for i, p in enumerate(("host", "device_insert", "device_dataflow"))},
        "mean_oper_per_column": float(np.mean([o["oper"].mean() for o in outs])),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": None},
        "gpu_launches": int(sum(1 for _ in outs)), "clocks": clk.summary(),
    }
    if args.mlp:
        mlp["final"] = consumer.train_eval(Pd, labels, split)
        out["mlp"] = mlp
    # e2e: the whole sequence again through the public API, each snapshot's P read back to pinned host memory
    # inside the timed region (the edge batch goes in from host arrays)
    indices2, degree2 = dyn.indices.copy(), dyn.degree.copy()
    G2 = api.Graph(dyn.indptr, indices2, row_len=degree2, degree=degree2.astype(np.float64), ctx=G.ctx)
    P2, R2 = torch.zeros_like(Xd), Xd.clone()
    api.feature_push(G2, L.IGN, P2, R2, eps, alpha=ALPHA, beta=beta, prec="fp32", tile_w=tw)
    P_host = torch.empty((n, F), dtype=torch.float32).pin_memory()
    torch.cuda.synchronize()
    e2e = []
    for s in range(snaps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        api.feature_update(G2, L.IGN, indices2, degree2, batches[s][0], batches[s][1], not mixed, P2, R2, Xd, eps,
                           alpha=ALPHA, beta=beta, prec="fp32", tile_w=tw)
        with torch.cuda.stream(stream):
            P_host.copy_(P2, non_blocking=True)
        e1.record(stream)
        e1.synchronize()
        e2e.append(e0.elapsed_time(e1))
    out["e2e"] = {"value": snaps / (sum(e2e) / 1e3), "unit": "snapshots/s",
                  "h2d_bytes_per_step": int(2 * 4 * batches[0][0].shape[0]), "d2h_bytes_per_step": int(n * F * 4)}
    G2.free()
    if not args.no_baselines:
        out.update(c5_oracle_check(dyn, X, batches, mixed, snapP, outs, beta, eps))
    print(json.dumps(out), flush=True)


C5_CHECK_COLS = 4


def c5_oracle_check(dyn, X, batches, mixed, snapP, outs, beta, eps):
    """accuracy: C5_CHECK_COLS FP32 columns after every snapshot against the FP64 oracle's synchronous update
    (the GPU's order); cpu_baseline: the oracle's port of the reference's FIFO update (instantGNNUpdateBatch,
    InstantGNN.py:298-329), one column per host thread on one snapshot, scaled to 128 columns."""
    from oracle import oracle as O
    n = dyn.n
    ip = dyn.indptr.astype(np.int64)
    threads = os.cpu_count() or 1
    Fs = max(C5_CHECK_COLS, min(threads, 16))
    ix, dg = dyn.indices.copy(), dyn.degree.copy()
    Xs = X[:, :Fs].astype(np.float64)
    Po, Ro = np.zeros((n, Fs)), Xs.copy()
    O.ign_sync(n, ip, ix, dg, ALPHA, eps, beta, Po, Ro)
    # CPU baseline: the reference's FIFO update of snapshot 0 on Fs columns in parallel
    ixb, dgb, Pb, Rb = ix.copy(), dg.copy(), Po.copy(), Ro.copy()
    t0 = time.perf_counter()
    O.ign_update(n, ip, ixb, dgb, ALPHA, eps, 1.0, Pb, Rb, Xs, batches[0][0], batches[0][1], beta,
                 "fwd" + ("" if mixed else "-insert"), sync=False)
    dt = time.perf_counter() - t0
    cpu = {"value": 1.0 / (dt * 128 / Fs), "unit": "snapshots/s", "cores": threads, "kind": "port",
           "sample": f"snapshot 0 on {Fs} of 128 columns in parallel (one per thread), {dt:.2f} s, "
                     f"scaled by 128/{Fs}"}
    # accuracy: the first C5_CHECK_COLS columns through every snapshot
    k = C5_CHECK_COLS
    Pa, Ra, Xa = Po[:, :k].copy(), Ro[:, :k].copy(), Xs[:, :k].copy()
    per = []
    for s, (us, vs) in enumerate(batches):
        _, oo = O.ign_update(n, ip, ix, dg, ALPHA, eps, 1.0, Pa, Ra, Xa, us, vs, beta,
                             "fwd" + ("" if mixed else "-insert"), sync=True)
        rel = np.abs(snapP[s] - Pa).sum(0) / np.abs(Pa).sum(0)
        od = np.abs(outs[s]["oper"][:k] - oo) / np.maximum(oo, 1)
        per.append({"snapshot": s, "rel_l1_max": float(rel.max()), "oper_rel_diff_max": float(od.max())})
    acc = {"vs": "FP64 oracle, synchronous update push (C port of instantGNNUpdateBatch's repair)",
           "columns": k, "snapshots": len(per), "rel_l1_max": max(p["rel_l1_max"] for p in per),
           "oper_rel_diff_max": max(p["oper_rel_diff_max"] for p in per), "per_snapshot": per}
    return {"accuracy": acc, "cpu_baseline": cpu}


def run_c1(args):
    """C1: PPR local GD in FP64 on the 100k-node Chung-Lu graph, 50 seeds at eps = 1e-6, checked against the
    oracle (operation counts exactly) and, for two seeds, against an FP64 global solve."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    from gde import _lib as L
    from gde import api, graphs
    from oracle import oracle as O
    g = graphs.chung_lu_100k()
    ctx = api.Context.get(local)
    G = api.Graph(g.indptr, g.indices, ctx=ctx)
    Q, alpha, eps = 50, 0.1, 1e-6
    deg = g.degree.astype(np.float64)
    stream = torch.cuda.ExternalStream(api.ctx_stream(ctx), device=f"cuda:{local}")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    x_dev = torch.empty((Q, g.n), dtype=torch.float64, device=f"cuda:{local}")
    r_dev = torch.empty((Q, g.n), dtype=torch.float64, device=f"cuda:{local}")

    def step(k, x_out=None, r_out=None, device_out=True):
        seeds = graphs.uniform_seeds(g, Q, seed=1 + 1000 * k)
        return api.solve(G, L.PPR, L.LOCAL_GD, seeds, eps, prec="fp64", alpha=alpha, tile_w=1,
                         x_out=x_dev if x_out is None else x_out, r_out=r_dev if r_out is None else r_out,
                         device_out=device_out)

    for w in range(args.warmup):
        step(10 + w)
    with ClockSampler(local) as clk:
        times, outs = _timed_steps(stream, flush, args.steps, lambda k: step(k))
    value = Q * len(times) * world / (sum(times) / 1e3)
    agg = {k: sum(o["stats"][k] for o in outs) for k in ("union_vol", "col_vol", "col_nodes", "kernel_ms")}
    # FP64: 4 B col_idx + 16 B residual RMW per edge, 48 B per active node
    achieved = (4 * agg["union_vol"] + 16 * agg["col_vol"] + 48 * agg["col_nodes"]) / (agg["kernel_ms"] / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    x_host = torch.empty((Q, g.n), dtype=torch.float64).pin_memory()
    e2e, _ = _timed_steps(stream, flush, max(1, args.e2e_steps), lambda k: step(200 + k, x_host, None, False), warm=1)
    out = {
        "metric": "PPR local GD queries/s, FP64, eps = 1e-6, 50 seeds, Chung-Lu 100k",
        "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sum(times) / len(times), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": "ppr_local_gd_fp64_50_seeds_chung_lu_100k", "n": g.n, "nnz": g.nnz,
                   "queries_per_step": Q, "alpha": alpha, "eps": eps, "l2": "512 MB buffer written between steps"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": None},
        "e2e": {"value": Q * len(e2e) / (sum(e2e) / 1e3), "unit": "queries/s", "h2d_bytes_per_step": Q * 12,
                "d2h_bytes_per_step": Q * g.n * 8},
        "gpu_launches": args.steps, "clocks": clk.summary(),
    }
    if not args.no_baselines:
        seeds = graphs.uniform_seeds(g, Q, seed=1 + 1000 * (args.steps - 1))
        threads = O.threads()
        t0 = time.perf_counter()
        oo, xo = O.ppr_gd_many(g.n, g.indptr, g.indices, deg, seeds, alpha, eps, keep_x=True, nthreads=threads)
        dt = time.perf_counter() - t0
        xg = x_dev.cpu().numpy()
        rg = r_dev.cpu().numpy()
        og = outs[-1]["oper"]
        truth = []
        for i in range(2):
            t_ = O.global_solve_ppr(g.indptr, g.indices, deg, int(seeds[i]), alpha)
            truth.append({"l1": float(np.abs(xg[i] - t_).sum()), "oracle_l1": float(np.abs(xo[i] - t_).sum()),
                          "max_r_over_d": float(np.max(np.abs(rg[i]) / deg))})
        out["accuracy"] = {"vs": "FP64 oracle (C port of ppr_gd local)", "queries": Q,
                           "oper_mismatches": int(np.sum(np.rint(og).astype(np.int64) != oo)),
                           "rel_l1_max": float((np.abs(xg - xo).sum(1) / np.abs(xo).sum(1)).max()),
                           "truth": {"vs": "FP64 global solve to 1e-15 (scipy)", "rows": truth,
                                     "stop_rule": eps * alpha}}
        out["cpu_baseline"] = {"value": Q / dt, "unit": "queries/s", "cores": threads, "kind": "port",
                               "sample": f"the step's 50 queries (ppr_gd local FP64, one per OpenMP thread), "
                                         f"{dt:.2f} s"}
    print(json.dumps(out), flush=True)


def run_c2_arms(args):
    """C2's four GPU arms on the 2.36M-node graph, 50 seeds at eps = 1e-7: local GD and local Chebyshev, each in
    FP64 and in FP32 residuals, beside the plain single-query kernel and the CPU ports."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    from gde import _lib as L
    from gde import api, graphs
    from oracle import oracle as O
    g = graphs.chung_lu_wikitalk_shape()
    ctx = api.Context.get(local)
    G = api.Graph(g.indptr, g.indices, ctx=ctx)
    Q = 50
    deg = g.degree.astype(np.float64)
    seeds = graphs.uniform_seeds(g, Q, seed=50)
    stream = torch.cuda.ExternalStream(api.ctx_stream(ctx), device=f"cuda:{local}")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    arms = []
    with ClockSampler(local) as clk:
        for method, mname in ((L.LOCAL_GD, "local_gd"), (L.LOCAL_CHEBY, "local_cheby")):
            for prec in ("fp64", "fp32"):
                def fn(k, method=method, prec=prec):
                    return api.solve(G, L.PPR, method, seeds, EPS, prec=prec, alpha=ALPHA, want_r=False,
                                     device_out=True)
                fn(0)
                times, outs = _timed_steps(stream, flush, max(1, args.steps // 2), fn)
                arms.append({"method": mname, "prec": prec, "queries_per_s": Q * len(times) / (sum(times) / 1e3),
                             "ms_per_step": sum(times) / len(times), "mean_oper": float(outs[-1]["oper"].mean()),
                             "x": outs[-1]["x"], "oper": outs[-1]["oper"]})
        # global GD in FP32 (ppr_gd_standard_gpu): every node in every round, so the dense phases (CHECK, the
        # dense PREP) stream over all n nodes; their share of the launch bounds what staging them could gain
        kg = 8
        def gfn(k):
            return api.solve(G, L.PPR, L.GLOBAL_GD, seeds[:kg], EPS, prec="fp32", alpha=ALPHA, want_r=False,
                             device_out=True)
        gfn(0)
        gt, gouts = _timed_steps(stream, flush, max(1, args.steps // 2), gfn)
        gst = gouts[-1]["stats"]
        rounds = int(np.max(gouts[-1]["rounds"]))
        tw = int(gst["tile_w"])
        # CHECK reads each node's residual row (tile_w FP32 values) and its FP64 degree once per round
        check_bytes = float(gst["tiles"]) * rounds * g.n * (4 * tw + 8)
        global_arm = {"method": "global_gd", "prec": "fp32", "queries": kg, "queries_per_s": kg * len(gt) / (sum(gt) / 1e3),
                      "ms_per_step": sum(gt) / len(gt), "rounds": rounds, "tile_w": tw, "tiles": int(gst["tiles"]),
                      "phase_ms": {k: float(gst[k + "_ms"]) for k in ("check", "prep", "scatter")},
                      "kernel_ms": float(gst["kernel_ms"]),
                      "check_gbs": check_bytes / max(float(gst["check_ms"]), 1e-9) / 1e6}
    xs = torch.zeros(g.n, dtype=torch.float32, device=f"cuda:{local}")
    api.plain_ppr_local(G, int(seeds[0]), ALPHA, EPS, x_out=xs)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in seeds[:16]:
        api.plain_ppr_local(G, int(s), ALPHA, EPS, x_out=xs)
    torch.cuda.synchronize()
    plain = 16 / (time.perf_counter() - t0)
    # FP64 oracle on 8 of the seeds: GD exactly, Chebyshev in the GPU's synchronous order
    k = 8
    threads = O.threads()
    t0 = time.perf_counter()
    oo, xo = O.ppr_gd_many(g.n, g.indptr, g.indices, deg, seeds[:k], ALPHA, EPS, keep_x=True, nthreads=threads)
    gd_cpu = k / (time.perf_counter() - t0)
    from concurrent.futures import ThreadPoolExecutor
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        che = list(ex.map(lambda s: O.cheby(g.n, g.indptr, g.indices, deg, int(s), ALPHA, EPS, True, sync=True),
                          seeds[:k]))
    ch_cpu = k / (time.perf_counter() - t0)
    for a in arms:
        x = a.pop("x")[:k].double().cpu().numpy()
        oper = a.pop("oper")[:k]
        if a["method"] == "local_gd":
            ref_x, ref_o = xo, oo.astype(np.float64)
        else:
            ref_x = np.stack([c[0] for c in che])
            ref_o = np.array([c[2] for c in che], np.float64)
        l1 = np.abs(x - ref_x).sum(1)
        a["accuracy"] = {"queries": k, "l1_max": float(l1.max()),
                         "rel_l1_max": float((l1 / np.abs(ref_x).sum(1)).max()),
                         "oper_rel_diff_max": float((np.abs(oper - ref_o) / ref_o).max())}
    best = arms[1]  # FP32 local GD
    out = {
        "metric": "PPR local GD / local Chebyshev queries/s, FP64 and FP32, eps = 1e-7, 50 seeds, Chung-Lu 2.36M",
        "value": best["queries_per_s"], "unit": "queries/s", "n_gpus": 1, "steps": max(1, args.steps // 2),
        "warmup": 1, "ms_per_step": best["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "ppr_local_gd_cheby_fp64_fp32_50_seeds_chung_lu_2.36M", "n": g.n, "nnz": g.nnz,
                   "queries_per_step": Q, "alpha": ALPHA, "eps": EPS, "value_arm": "local_gd fp32"},
        "arms": arms, "global_gd": global_arm,
        "plain_gpu": {"value": plain, "unit": "queries/s", "sample": "16 queries"},
        "cpu_baseline": {"value": gd_cpu, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": f"{k} of the seeds, ppr_gd local FP64, one per thread; local Chebyshev "
                                   f"(synchronous order) {ch_cpu:.1f} q/s"},
        "gpu_launches": 4 * max(1, args.steps // 2), "clocks": clk.summary(),
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "c1":
        run_c1(args)
    elif args.workload == "c2arms":
        run_c2_arms(args)
    elif args.workload == "c3":
        run_c3(args)
    elif args.workload == "c4":
        run_c4(args)
    elif args.workload == "c5":
        run_c5(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
