"""Seeded synthetic graphs standing in for the reference's datasets.

The reference solves on SNAP/OGB graphs (wiki-talk, ogbn-arxiv) that it
preprocesses into scipy CSR ``.npz`` files (``data_process.py:29-45``:
largest connected component, relabelled, symmetric, no self-loops) and, for
the InstantGNN experiment, into a *padded* CSR with slack slots
(``data_process_GNN.py:93-171``).  Those datasets are not available, so this
module generates graphs of the same shape:

* ``chung_lu``  -- undirected Chung-Lu graph with power-law expected degrees;
* ``rmat``      -- R-MAT (Kronecker) graph;
* ``dynamic_padded`` -- the InstantGNN dynamic-graph layout: a padded CSR that
  holds the initial graph (spanning forest + kept edges) with slack for the
  edges that are re-inserted over ``snapshots`` batches.

Every generator is deterministic in its seed.  Static graphs have degree-0
nodes dropped and relabelled, because the reference's global and GPU loops
never terminate on an isolated node (``eps*alpha*0 <= |0|`` is always true,
``ppr_solver.py:65``, ``:139``).
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np


@dataclasses.dataclass
class CSRGraph:
    """Symmetric CSR adjacency: neighbours of ``u`` are ``indices[indptr[u]:indptr[u+1]]``."""

    indptr: np.ndarray   # int64 [n+1]
    indices: np.ndarray  # int32 [nnz]
    name: str = ""

    @property
    def n(self) -> int:
        return int(self.indptr.shape[0] - 1)

    @property
    def nnz(self) -> int:
        return int(self.indices.shape[0])

    @property
    def degree(self) -> np.ndarray:
        """Integer degree (row length); the reference's ``adj.sum(1)``."""
        return np.diff(self.indptr).astype(np.int64)


def _csr_from_undirected(n: int, a: np.ndarray, b: np.ndarray, drop_isolated: bool) -> tuple[CSRGraph, np.ndarray]:
    """Symmetrise, dedup and drop self-loops of an undirected edge list; build CSR.

    Returns the graph and the old->new relabelling (-1 for dropped nodes).
    """
    keep = a != b
    a = a[keep].astype(np.int64)
    b = b[keep].astype(np.int64)
    lo = np.minimum(a, b)
    hi = np.maximum(a, b)
    key = np.unique(lo * n + hi)
    lo = key // n
    hi = key % n
    relabel = np.arange(n, dtype=np.int64)
    if drop_isolated:
        deg = np.bincount(lo, minlength=n) + np.bincount(hi, minlength=n)
        alive = deg > 0
        relabel = np.full(n, -1, dtype=np.int64)
        relabel[alive] = np.arange(int(alive.sum()), dtype=np.int64)
        lo = relabel[lo]
        hi = relabel[hi]
        n = int(alive.sum())
    src = np.concatenate([lo, hi])
    dst = np.concatenate([hi, lo])
    order = np.lexsort((dst, src))
    src = src[order]
    dst = dst[order]
    indptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(src, minlength=n), out=indptr[1:])
    return CSRGraph(indptr=indptr, indices=dst.astype(np.int32)), relabel


def chung_lu(n: int, exponent: float, mean_degree: float, max_degree: float, seed: int,
             drop_isolated: bool = True, name: str = "") -> CSRGraph:
    """Undirected Chung-Lu graph with power-law expected degrees.

    Weights ``w_i = (1-U)^{-1/(exponent-1)}`` are rescaled to ``mean_degree``
    and capped at ``max_degree``; ``sum(w)/2`` edges are drawn with both
    endpoints proportional to ``w``; the result is symmetrised, deduplicated,
    stripped of self-loops and (by default) of degree-0 nodes.
    """
    rng = np.random.default_rng(seed)
    u = rng.random(n)
    w = (1.0 - u) ** (-1.0 / (exponent - 1.0))
    w *= mean_degree / w.mean()
    np.minimum(w, max_degree, out=w)
    m = int(round(w.sum() / 2.0))
    p = w / w.sum()
    cdf = np.cumsum(p)
    cdf[-1] = 1.0
    a = np.searchsorted(cdf, rng.random(m), side="right")
    b = np.searchsorted(cdf, rng.random(m), side="right")
    np.minimum(a, n - 1, out=a)
    np.minimum(b, n - 1, out=b)
    g, _ = _csr_from_undirected(n, a, b, drop_isolated)
    g.name = name or f"chung_lu_n{n}_e{exponent}_s{seed}"
    return g


def rmat(scale: int, edge_factor: int, a: float, b: float, c: float, seed: int,
         drop_isolated: bool = True, name: str = "", chunk: int = 1 << 23) -> CSRGraph:
    """R-MAT graph on ``2**scale`` nodes with ``edge_factor * 2**scale`` CSR entries (before dedup).

    ``edge_factor * 2**scale / 2`` undirected edges are sampled; symmetrising
    gives ``edge_factor`` CSR entries per node before duplicates and
    self-loops are dropped (scale 22, factor 16: ~67M entries).
    """
    rng = np.random.default_rng(seed)
    n = 1 << scale
    m = edge_factor * n // 2
    srcs = []
    dsts = []
    ab = a + b
    abc = a + b + c
    for start in range(0, m, chunk):
        k = min(chunk, m - start)
        s = np.zeros(k, dtype=np.int64)
        d = np.zeros(k, dtype=np.int64)
        for _ in range(scale):
            r = rng.random(k)
            s <<= 1
            d <<= 1
            s += (r >= ab)
            d += ((r >= a) & (r < ab)) | (r >= abc)
        srcs.append(s)
        dsts.append(d)
    g, _ = _csr_from_undirected(n, np.concatenate(srcs), np.concatenate(dsts), drop_isolated)
    g.name = name or f"rmat_s{scale}_ef{edge_factor}_s{seed}"
    return g


@dataclasses.dataclass
class DynamicGraph:
    """Padded CSR in the reference's InstantGNN layout (``data_process_GNN.py:93-171``).

    ``indptr`` is the full graph's row pointer (capacity of each row); the
    live neighbours of ``u`` are ``indices[indptr[u]:indptr[u]+degree[u]]`` and
    the slack slots hold the sentinel ``n``.  ``Us[s], Vs[s]`` are the
    undirected edges re-inserted at snapshot ``s``.
    """

    indptr: np.ndarray   # int64 [n+1]
    indices: np.ndarray  # int32 [capacity]
    degree: np.ndarray   # int64 [n]
    Us: np.ndarray       # int32 [snapshots, batch]
    Vs: np.ndarray       # int32 [snapshots, batch]
    name: str = ""

    @property
    def n(self) -> int:
        return int(self.indptr.shape[0] - 1)


def dynamic_padded(g: CSRGraph, delnum: int, snapshots: int, seed: int) -> DynamicGraph:
    """Initial graph = random spanning forest + all but ``delnum`` other edges.

    Follows the construction of ``data_process_GNN.py``: full-graph row
    capacity, spanning-forest edges placed first (Kruskal over shuffled
    edges), then the kept non-forest edges, slack filled with ``n``; the
    ``delnum`` held-out edges are shuffled into ``snapshots`` equal batches.
    """
    rng = np.random.default_rng(seed)
    n = g.n
    indptr = g.indptr.copy()
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(indptr))
    dst = g.indices.astype(np.int64)
    und = src < dst
    eu = src[und]
    ev = dst[und]
    m = eu.shape[0]
    perm = rng.permutation(m)
    eu = eu[perm]
    ev = ev[perm]
    # Kruskal over the shuffled edge order picks the minimum spanning forest
    # under weight = position in that order; scipy computes the same forest.
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import minimum_spanning_tree
    wgt = np.arange(1, m + 1, dtype=np.float64)
    mst = minimum_spanning_tree(coo_matrix((wgt, (eu, ev)), shape=(n, n)).tocsr()).tocoo()
    in_forest = np.zeros(m, dtype=bool)
    in_forest[mst.data.astype(np.int64) - 1] = True
    rest = np.nonzero(~in_forest)[0]
    rest = rest[rng.permutation(rest.shape[0])]
    delnum = min(delnum, rest.shape[0])
    kept = rest[: rest.shape[0] - delnum]
    held = rest[rest.shape[0] - delnum:]
    init = np.concatenate([np.nonzero(in_forest)[0], kept])
    degree = np.zeros(n, dtype=np.int64)
    indices = np.full(g.nnz, n, dtype=np.int32)
    # Place edges in order: forest first, then kept edges (row order = insertion order).
    a = eu[init]
    b = ev[init]
    ends = np.concatenate([np.stack([a, b], 1), np.stack([b, a], 1)], 0)
    order_key = np.concatenate([np.arange(init.shape[0]) * 2, np.arange(init.shape[0]) * 2 + 1])
    ends = ends[np.argsort(order_key, kind="stable")]
    # rank of each (row, entry) within its row in insertion order
    rows = ends[:, 0]
    o = np.argsort(rows, kind="stable")
    rows_sorted = rows[o]
    counts = np.bincount(rows_sorted, minlength=n)
    starts = np.zeros(n, dtype=np.int64)
    np.cumsum(counts[:-1], out=starts[1:])
    rank = np.arange(rows_sorted.shape[0]) - starts[rows_sorted]
    pos = indptr[rows_sorted] + rank
    indices[pos] = ends[o, 1].astype(np.int32)
    degree[:] = counts
    batch = held.shape[0] // snapshots
    sel = held[: batch * snapshots]
    Us = eu[sel].reshape(snapshots, batch).astype(np.int32)
    Vs = ev[sel].reshape(snapshots, batch).astype(np.int32)
    return DynamicGraph(indptr=indptr, indices=indices, degree=degree, Us=Us, Vs=Vs,
                        name=f"{g.name}_dyn_del{delnum}_snap{snapshots}")


# ---------------------------------------------------------------------------
# Named workloads (sizes of the five benchmark configurations)
# ---------------------------------------------------------------------------

def _cache_dir() -> str:
    d = os.environ.get("GDE_GRAPH_CACHE") or os.path.join(
        os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), ".graph_cache")
    os.makedirs(d, exist_ok=True)
    return d


def _cached(name: str, make):
    path = os.path.join(_cache_dir(), name + ".npz")
    if os.path.exists(path):
        z = np.load(path)
        return CSRGraph(indptr=z["indptr"], indices=z["indices"], name=name)
    g = make()
    g.name = name
    tmp = path + f".{os.getpid()}.tmp.npz"
    np.savez(tmp, indptr=g.indptr, indices=g.indices)
    os.replace(tmp, path)
    return g


def chung_lu_100k() -> CSRGraph:
    """n=100,000, exponent 2.1, mean 10, max 2,000, seed 0 (degree-0 nodes dropped)."""
    return _cached("cl100k", lambda: chung_lu(100_000, 2.1, 10.0, 2_000.0, seed=0))


def chung_lu_wikitalk_shape() -> CSRGraph:
    """The wiki-talk shape: ~2.36M nodes, ~9.36M CSR entries, max degree ~62k, 60% degree-1.

    A pure exponent-2.0 Chung-Lu graph leaves too many isolated nodes to reach
    2.39M live nodes at mean degree 3.9, so the weights use exponent 2.1 over
    5.65M candidate nodes; after dropping degree-0 nodes this gives n=2,364,073,
    nnz=9,355,158, mean degree 3.96.
    """
    return _cached("cl2p36m", lambda: chung_lu(5_650_000, 2.1, 1.92, 100_000.0, seed=0))


def rmat_scale22() -> CSRGraph:
    """R-MAT scale 22, edge factor 16, (a,b,c) = (0.57, 0.19, 0.19), symmetrised."""
    return _cached("rmat22", lambda: rmat(22, 16, 0.57, 0.19, 0.19, seed=0))


def chung_lu_arxiv_shape() -> CSRGraph:
    """n=169,343, ~1.17M undirected edges, exponent 2.3; isolated nodes are kept."""
    return _cached("cl169k", lambda: chung_lu(169_343, 2.3, 14.5, 20_000.0, seed=0, drop_isolated=False))


def uniform_seeds(g: CSRGraph, count: int, seed: int) -> np.ndarray:
    """``count`` seeds drawn uniformly from the nodes with degree >= 1."""
    rng = np.random.default_rng(seed)
    cand = np.nonzero(np.diff(g.indptr) > 0)[0]
    return cand[rng.integers(0, cand.shape[0], size=count)].astype(np.int32)
