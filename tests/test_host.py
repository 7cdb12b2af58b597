"""Host-side logic of the Python mirror: rescale, sampling, graph storage,
LG reading, argument errors and generators.  No GPU needed."""
import numpy as np
import pytest

import lgbc
from lgbc import generators as G
from lgbc.centrality import _sources0
from oracle import oracle


@pytest.mark.parametrize("n", [0, 1, 2, 3, 50, 46341, 46342, 10**6])
@pytest.mark.parametrize("normalize", [False, True])
@pytest.mark.parametrize("directed", [False, True])
@pytest.mark.parametrize("kfrac", [0.0, 0.3, 1.0])
def test_rescale_matches_oracle(n, normalize, directed, kfrac):
    # src/centrality/betweenness.jl:136-160, bit for bit
    rng = np.random.default_rng(n)
    raw = rng.random(n) * 100
    k = int(n * kfrac)
    a = raw.copy()
    lgbc._rescale_(a, n, normalize, directed, k)
    b = oracle.rescale(raw, n, normalize, directed, k)
    assert np.array_equal(a, b)


def test_sample_distinct_and_argument_error():
    # src/utils.jl:12-28 / :43
    s = lgbc.sample(range(1, 101), 100, rng=1)
    assert sorted(s) == list(range(1, 101))
    s = lgbc.sample(range(1, 1001), 50, rng=2)
    assert len(set(s)) == 50 and all(1 <= x <= 1000 for x in s)
    with pytest.raises(lgbc.ArgumentError):
        lgbc.sample(range(1, 4), 4)
    a = list(range(1, 11))
    lgbc.sample_(a, 3, rng=3)
    assert sorted(a) == list(range(1, 11))  # sample! permutes in place


def test_graph_storage_matches_fadjlist():
    # sorted unique lists; a self-loop stored once (simplegraph.jl:445-461)
    g = lgbc.SimpleGraph(4)
    for u, v in [(1, 2), (2, 1), (3, 3), (4, 2), (1, 2)]:
        g.add_edge(u, v)
    rp, ci = g.csr()
    assert rp.tolist() == [0, 1, 3, 4, 5]
    assert ci.tolist() == [1, 0, 3, 2, 1]
    assert g.ne() == 3 and g.degree(3) == 1 and g.degree(2) == 2
    d = lgbc.SimpleDiGraph(3)
    for u, v in [(1, 2), (2, 3), (3, 3)]:
        d.add_edge(u, v)
    assert d.degree(3) == 3 and d.degree(1) == 1 and d.ne() == 3
    assert d.inneighbors(3).tolist() == [2, 3]
    assert d.outneighbors(2).tolist() == [3]


def test_loadgraph_golden(golden_graph):
    assert golden_graph.is_directed()
    assert golden_graph.nv() == 50 and golden_graph.ne() == 500
    rp, ci = golden_graph.csr()
    for v in range(50):
        row = ci[rp[v]:rp[v + 1]]
        assert np.all(np.diff(row) > 0)


def test_source_validation():
    g = lgbc.SimpleGraph.from_edges(3, [(1, 2)])
    assert _sources0(g, [1, 3]).tolist() == [0, 2]
    assert _sources0(g, range(1, 4)).tolist() == [0, 1, 2]
    with pytest.raises(lgbc.BoundsError):
        _sources0(g, [0])
    with pytest.raises(lgbc.BoundsError):
        _sources0(g, [4])


def test_non_unit_weights_are_a_method_error():
    g = lgbc.SimpleGraph.from_edges(3, [(1, 2)])
    with pytest.raises(lgbc.MethodError):
        lgbc.betweenness_centrality(g, None, np.ones((3, 3)))
    with pytest.raises(lgbc.ArgumentError):
        lgbc.betweenness_centrality(g, 4)  # k > n, raised by sample before any GPU call


def test_generators_follow_reference_semantics():
    g = G.erdos_renyi_nm(1000, 4000, seed=5)
    assert g.nv() == 1000 and g.ne() == 4000
    rp, ci = g.csr()
    src = np.repeat(np.arange(1000), np.diff(rp))
    assert not np.any(src == ci)  # no self-loops
    for n in (200, 1000, 5000):
        b = G.barabasi_albert(n, 3, seed=n)
        assert b.ne() == 3 * (n - 3)  # randgraphs.jl:449-512 adds k edges per new vertex
        assert np.all(b.degrees()[3:] >= 3)
    r = G.rmat(12, 16, seed=1)
    rp, ci = r.csr()
    assert len(ci) == 2 * r.ne()
    src = np.repeat(np.arange(r.nv()), np.diff(rp))
    assert not np.any(src == ci)
    d = G.rmat(12, 16, seed=1, directed=True)
    assert d.ne() == len(d.csr()[1]) == len(d.in_csr()[1])
    # same seed, same graph; different seed, different graph
    assert np.array_equal(G.rmat(10, 8, seed=4).csr()[1], G.rmat(10, 8, seed=4).csr()[1])
    assert not np.array_equal(G.rmat(10, 8, seed=4).csr()[1], G.rmat(10, 8, seed=5).csr()[1])
