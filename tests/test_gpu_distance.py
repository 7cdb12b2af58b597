"""GPU parity of the distance metrics (multi-source BFS statistics) against
the oracle and the reference's golden vector."""
import warnings

import numpy as np
import pytest

import lgbc
import lgbc.generators as gen
from conftest import golden_path
from oracle import oracle

pytestmark = pytest.mark.gpu


def _graphs():
    rng = np.random.default_rng(3)
    e = rng.integers(1, 301, size=(700, 2))
    e = e[e[:, 0] != e[:, 1]]
    yield lgbc.SimpleGraph.from_edges(300, [tuple(x) for x in e.tolist()])
    yield lgbc.SimpleDiGraph.from_edges(300, [tuple(x) for x in e.tolist()])
    yield gen.rmat(10, 8, seed=4)
    yield gen.barabasi_albert(500, 2, seed=5)
    yield lgbc.SimpleGraph.from_edges(200, [(i, i + 1) for i in range(1, 200)])  # path


@pytest.mark.parametrize("idx", range(5))
def test_distance_stats_match_oracle(idx):
    g = list(_graphs())[idx]
    rp, ci = g.csr()
    n = g.nv()
    src = np.arange(n, dtype=np.int32)
    reached, dsum, dmax = lgbc.distance.distance_stats(g, src)
    for s in range(0, n, max(1, n // 60)):
        d = oracle.gdistances(rp, ci, [s]).astype(np.int64)
        ok = d != oracle.UNREACHED32
        assert reached[s] == ok.sum() and dsum[s] == d[ok].sum() and dmax[s] == d[ok].max()


@pytest.mark.parametrize("idx", range(5))
def test_closeness_radiality_eccentricity_match_oracle(idx):
    g = list(_graphs())[idx]
    rp, ci = g.csr()
    for norm in (True, False):
        assert np.array_equal(lgbc.closeness_centrality(g, normalize=norm),
                              oracle.closeness(rp, ci, g.degrees(), normalize=norm))
    assert np.array_equal(lgbc.radiality_centrality(g), oracle.radiality(rp, ci))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        assert np.array_equal(lgbc.eccentricity(g), oracle.eccentricity(rp, ci))
        assert np.array_equal(lgbc.Parallel.eccentricity(g), oracle.eccentricity(rp, ci))
    assert np.array_equal(lgbc.Parallel.radiality_centrality(g, parallel="threads"),
                          oracle.radiality(rp, ci))


def test_radiality_golden(golden_graph):
    want = np.loadtxt(golden_path("graph-50-500-rc.txt"), delimiter=",")
    assert np.array_equal(lgbc.radiality_centrality(golden_graph), want)


def test_known_answers_and_measures():
    g = lgbc.SimpleGraph.from_edges(5, [(1, 2), (2, 3), (3, 4), (1, 4), (4, 5)])
    np.testing.assert_allclose(lgbc.radiality_centrality(g), [5 / 6, 3 / 4, 5 / 6, 11 / 12, 2 / 3])
    d = lgbc.SimpleDiGraph.from_edges(4, [(1, 2), (2, 3), (1, 3), (3, 4)])
    assert lgbc.closeness_centrality(d).tolist() == [0.75, 0.4444444444444444,
                                                     0.3333333333333333, 0.0]
    path5 = lgbc.SimpleGraph.from_edges(5, [(i, i + 1) for i in range(1, 5)])
    assert lgbc.eccentricity(path5).tolist() == [4, 3, 2, 3, 4]
    assert lgbc.eccentricity(path5, 3) == 2
    assert lgbc.diameter(path5) == 4 and lgbc.radius(path5) == 2
    assert lgbc.periphery(path5) == [1, 5] and lgbc.center(path5) == [3]
    with pytest.warns(UserWarning):
        lgbc.eccentricity(lgbc.SimpleGraph.from_edges(3, [(1, 2)]))
    with pytest.raises(lgbc.MethodError):
        lgbc.closeness_centrality(g, np.ones((5, 5)))
