"""GPU parity of bfs_parents / bfs_tree / has_path against the oracle."""
import numpy as np
import pytest

import lgbc
import lgbc.generators as gen
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_known_answers():
    g5 = lgbc.SimpleDiGraph.from_edges(4, [(1, 2), (2, 3), (1, 3), (3, 4)])
    assert lgbc.bfs_parents(g5, 1).tolist() == [1, 1, 1, 3]
    z = lgbc.bfs_tree(g5, 1)
    assert z.nv() == 4 and z.ne() == 3 and not z.has_edge(2, 3)
    house = lgbc.SimpleGraph.from_edges(5, [(1, 2), (1, 3), (2, 4), (3, 4), (3, 5), (4, 5)])
    p = lgbc.bfs_parents(house, 1)
    t = lgbc.bfs_tree(house, 1)
    assert t.ne() < t.nv() and t.is_directed()
    assert lgbc.tree(p).csr()[1].tolist() == t.csr()[1].tolist()
    zp = lgbc.Parallel.bfs_tree(g5, 1)
    assert zp.ne() == 3


@pytest.mark.parametrize("kind", ["rmat", "rmat_dir", "ba", "sparse"])
def test_bfs_parents_match_oracle(kind):
    rng = np.random.default_rng(5)
    if kind == "rmat":
        g = gen.rmat(12, 8, seed=3)
    elif kind == "rmat_dir":
        g = gen.rmat(12, 8, seed=4, directed=True)
    elif kind == "ba":
        g = gen.barabasi_albert(3000, 2, seed=6)
    else:
        e = rng.integers(1, 2001, size=(1500, 2))
        g = lgbc.SimpleGraph.from_edges(2000, [tuple(x) for x in e[e[:, 0] != e[:, 1]].tolist()])
    rp, ci = g.csr()
    irp, ici = g.in_csr()
    deg = g.degrees()
    for s in rng.choice(np.flatnonzero(deg > 0), 4, replace=False).tolist():
        want = oracle.bfs_parents(rp, ci, s) + 1
        assert np.array_equal(lgbc.bfs_parents(g, s + 1).astype(np.int64), want)
        if g.is_directed():
            want_in = oracle.bfs_parents(irp, ici, s) + 1
            assert np.array_equal(lgbc.bfs_parents(g, s + 1, dir="in").astype(np.int64), want_in)


def test_has_path_matches_oracle():
    g = gen.rmat(10, 4, seed=8, directed=True)
    rp, ci = g.csr()
    rng = np.random.default_rng(2)
    for _ in range(30):
        u, v = (int(x) for x in rng.integers(0, g.nv(), 2))
        ex = rng.integers(0, g.nv(), 20).tolist()
        assert lgbc.has_path(g, u + 1, v + 1, exclude_vertices=[x + 1 for x in ex]) == \
            oracle.has_path(rp, ci, u, v, ex)
        assert lgbc.has_path(g, u + 1, v + 1) == oracle.has_path(rp, ci, u, v)
    assert lgbc.has_path(g, 3, 3)
    assert not lgbc.has_path(g, 3, 3, exclude_vertices=[3])
