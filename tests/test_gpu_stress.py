"""GPU parity of stress centrality against the oracle (bit-exact Int64,
wrapping overflow included) and the reference's golden vector."""
import numpy as np
import pytest

import lgbc
import lgbc.generators as gen
from conftest import golden_path
from oracle import oracle

pytestmark = pytest.mark.gpu


def _args(g):
    rp, ci = g.csr()
    kw = dict(directed=g.is_directed())
    if g.is_directed():
        irp, ici = g.in_csr()
        kw.update(in_rowptr=irp, in_colidx=ici)
    return rp, ci, kw


def test_stress_golden(golden_graph):
    want = np.loadtxt(golden_path("graph-50-500-sc.txt"), delimiter=",").astype(np.int64)
    assert np.array_equal(lgbc.stress_centrality(golden_graph), want)
    assert np.array_equal(lgbc.Parallel.stress_centrality(golden_graph, parallel="threads"), want)


def test_stress_known_answers():
    g = lgbc.SimpleGraph.from_edges(5, [(1, 2), (2, 3), (3, 4), (1, 4), (4, 5)])
    assert lgbc.stress_centrality(g).tolist() == [4, 2, 4, 10, 0]
    assert lgbc.stress_centrality(lgbc.SimpleGraph.from_edges(3, [(1, 2), (1, 3)])).tolist() == [2, 0, 0]
    x = lgbc.stress_centrality(g, 3, rng=np.random.default_rng(1))
    assert x.shape == (5,)


@pytest.mark.parametrize("kind", ["er", "er_dir", "rmat", "ba", "hubs"])
def test_stress_matches_oracle(kind):
    rng = np.random.default_rng(7)
    if kind in ("er", "er_dir"):
        e = rng.integers(1, 401, size=(1600, 2))
        e = [tuple(x) for x in e[e[:, 0] != e[:, 1]].tolist()]
        g = (lgbc.SimpleDiGraph if kind == "er_dir" else lgbc.SimpleGraph).from_edges(400, e)
    elif kind == "rmat":
        g = gen.rmat(11, 16, seed=9)
    elif kind == "ba":
        g = gen.barabasi_albert(1500, 3, seed=2)
    else:  # two hubs of degree 700 share neighbours: hub items on both sweeps
        e = [(1, v) for v in range(3, 703)] + [(2, v) for v in range(3, 703)] + [(703, 1)]
        g = lgbc.SimpleGraph.from_edges(703, e)
    rp, ci, kw = _args(g)
    src = np.arange(g.nv(), dtype=np.int32)[::3].copy()
    src = np.concatenate([src, src[:5]])  # repeats count twice
    want = oracle.stress(rp, ci, src, **kw)
    got = lgbc.stress_centrality(g, src + 1)
    assert np.array_equal(got, want)


def test_stress_wraps_like_julia():
    # 40 x 40 grid: DAG path counts far beyond 2^64, so the Int64 sums wrap
    n = 40
    edges = [(r * n + c + 1, r * n + c + 2) for r in range(n) for c in range(n - 1)]
    edges += [(r * n + c + 1, (r + 1) * n + c + 1) for r in range(n - 1) for c in range(n)]
    g = lgbc.SimpleGraph.from_edges(n * n, edges)
    rp, ci = g.csr()
    src = np.array([0, 39, 820, 1599], np.int32)
    assert np.array_equal(lgbc.stress_centrality(g, src + 1), oracle.stress(rp, ci, src))
