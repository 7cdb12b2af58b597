"""CPU pins of the oracle's distance metrics against the reference's golden
vector and known answers (test/centrality/{radiality,closeness}.jl,
src/centrality/*.jl doc examples, src/distance.jl doc examples)."""
import numpy as np
import pytest

import lgbc
from conftest import golden_path
from oracle import oracle


def _cycle4_plus():
    # cycle_graph(4); add_vertex!; add_edge!(4, 5)
    return lgbc.SimpleGraph.from_edges(5, [(1, 2), (2, 3), (3, 4), (1, 4), (4, 5)])


def test_radiality_golden(golden_graph):
    rp, ci = golden_graph.csr()
    want = np.loadtxt(golden_path("graph-50-500-rc.txt"), delimiter=",")
    assert np.array_equal(oracle.radiality(rp, ci), want)


def test_radiality_known_answers():
    g = _cycle4_plus()
    rp, ci = g.csr()
    np.testing.assert_allclose(oracle.radiality(rp, ci), [5 / 6, 3 / 4, 5 / 6, 11 / 12, 2 / 3])
    star = lgbc.SimpleGraph.from_edges(4, [(1, 2), (1, 3), (1, 4)])
    np.testing.assert_allclose(oracle.radiality(*star.csr()), [1.0, 2 / 3, 2 / 3, 2 / 3])
    path3 = lgbc.SimpleGraph.from_edges(3, [(1, 2), (2, 3)])
    np.testing.assert_allclose(oracle.radiality(*path3.csr()), [0.75, 1.0, 0.75])


def test_closeness_known_answers():
    g = lgbc.SimpleDiGraph.from_edges(4, [(1, 2), (2, 3), (1, 3), (3, 4)])
    rp, ci = g.csr()
    assert oracle.closeness(rp, ci, g.degrees(), normalize=False).tolist() == \
        [0.75, 0.6666666666666666, 1.0, 0.0]
    assert oracle.closeness(rp, ci, g.degrees()).tolist() == \
        [0.75, 0.4444444444444444, 0.3333333333333333, 0.0]
    g5 = lgbc.SimpleGraph.from_edges(5, [(1, 2)])
    z = oracle.closeness(*g5.csr(), g5.degrees())
    assert z[0] == z[1] == 0.25 and z[2] == z[3] == z[4] == 0.0
    star = lgbc.SimpleGraph.from_edges(5, [(1, v) for v in range(2, 6)])
    np.testing.assert_array_equal(oracle.closeness(*star.csr(), star.degrees()),
                                  [1.0] + [0.5714285714285714] * 4)


def test_eccentricity_known_answers():
    # src/distance.jl:44-56 doc example: a three-vertex graph with edges 1-2, 2-3
    g = lgbc.SimpleGraph.from_edges(3, [(1, 2), (2, 3)])
    rp, ci = g.csr()
    assert oracle.eccentricity(rp, ci).tolist() == [2, 1, 2]
    assert oracle.eccentricity(rp, ci, [0, 1]).tolist() == [2, 1]
    d = lgbc.SimpleDiGraph.from_edges(3, [(1, 2)])
    assert oracle.eccentricity(*d.csr()).tolist() == [np.iinfo(np.int64).max] * 3


def test_radiality_wraps_like_julia_int64():
    # two components: every distance vector holds typemax(Int), whose Int64
    # sums wrap around exactly as Julia's do
    g = lgbc.SimpleGraph.from_edges(5, [(1, 2), (2, 3), (4, 5)])
    rp, ci = g.csr()
    r = oracle.radiality(rp, ci)
    with np.errstate(over="ignore"):
        s = np.int64(2**63 - 1) * np.int64(2) + np.int64(3)
    assert r[0] == ((float(2**63 - 1) + 1) - float(s) / 4) / float(2**63 - 1)


def test_stress_golden_and_known_answers(golden_graph):
    rp, ci = golden_graph.csr()
    irp, ici = golden_graph.in_csr()
    want = np.loadtxt(golden_path("graph-50-500-sc.txt"), delimiter=",").astype(np.int64)
    got = oracle.stress(rp, ci, directed=True, in_rowptr=irp, in_colidx=ici)
    assert np.array_equal(got, want)
    assert oracle.stress(*_cycle4_plus().csr()).tolist() == [4, 2, 4, 10, 0]
    star = lgbc.SimpleGraph.from_edges(3, [(1, 2), (1, 3)])
    assert oracle.stress(*star.csr()).tolist() == [2, 0, 0]
    c4 = lgbc.SimpleGraph.from_edges(4, [(1, 2), (2, 3), (3, 4), (1, 4)])
    assert oracle.stress(*c4.csr()).tolist() == [2, 2, 2, 2]


def test_bfs_parents_oracle_known_answers():
    g5 = lgbc.SimpleDiGraph.from_edges(4, [(1, 2), (2, 3), (1, 3), (3, 4)])
    rp, ci = g5.csr()
    assert (oracle.bfs_parents(rp, ci, 0) + 1).tolist() == [1, 1, 1, 3]
    # house graph (smallgraph(:house)): 1-2, 1-3, 2-4, 3-4, 3-5, 4-5
    house = lgbc.SimpleGraph.from_edges(5, [(1, 2), (1, 3), (2, 4), (3, 4), (3, 5), (4, 5)])
    p = oracle.bfs_parents(*house.csr(), 0) + 1
    assert p.tolist() == [1, 1, 1, 2, 3]
    t = lgbc.tree(p)
    assert t.is_directed() and t.ne() < t.nv()
    assert oracle.has_path(rp, ci, 0, 3) and not oracle.has_path(rp, ci, 3, 0)
    assert not oracle.has_path(rp, ci, 0, 3, exclude=[2])
