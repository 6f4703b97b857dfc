"""Replica sharding across ranks (host logic, gloo on CPU, world_size 2).

The GPU solve is replaced by the oracle here: what is tested is that every
query is solved by exactly one rank and that the gathered per-query results
come back complete and in query order.
"""
import os
import socket

import numpy as np
import pytest

from gde import graphs, replicas


def test_shard_bounds_partition():
    for n in (0, 1, 7, 512, 1000):
        for world in (1, 2, 3, 8):
            cuts = [replicas.shard_bounds(n, world, r) for r in range(world)]
            assert cuts[0][0] == 0 and cuts[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(cuts, cuts[1:]))
            sizes = [hi - lo for lo, hi in cuts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard_bounds(10, 2, 2)


def _oracle_solve(seeds, eps, g=None, alpha=0.1):
    from oracle import oracle as O
    deg = g.degree.astype(np.float64)
    opers, rounds = [], []
    for s, e in zip(seeds, eps):
        _, _, o = O.ppr_gd(g.n, g.indptr, g.indices, deg, int(s), alpha, float(e), True)
        opers.append(o)
        rounds.append(int(s))  # stands in for a per-query value that identifies the query
    return {"oper": np.array(opers), "rounds": np.array(rounds)}


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        g = graphs.chung_lu(400, 2.1, 6.0, 60.0, seed=4)
        seeds = graphs.uniform_seeds(g, 11, seed=3)
        eps = np.full(11, 1e-5)
        out = replicas.solve_sharded(seeds, eps, _oracle_solve, g=g)
        q.put((rank, out["lo"], out["hi"], out["oper"].tolist(), out["rounds"].tolist()))
    finally:
        dist.destroy_process_group()


def test_solve_sharded_gloo_two_ranks():
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    g = graphs.chung_lu(400, 2.1, 6.0, 60.0, seed=4)
    seeds = graphs.uniform_seeds(g, 11, seed=3)
    full = _oracle_solve(seeds, np.full(11, 1e-5), g=g)
    assert (res[0][1], res[0][2], res[1][1], res[1][2]) == (0, 5, 5, 11)
    for _, _, _, oper, rounds in res:
        np.testing.assert_array_equal(oper, full["oper"])
        np.testing.assert_array_equal(rounds, seeds)
