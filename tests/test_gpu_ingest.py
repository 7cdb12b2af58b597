"""Graph ingest on the device (lgbc_graph_create_from_edges): the CSR equals
the add_edge! storage built on the host, for undirected and directed graphs,
duplicates, self-loops, isolated vertices and an empty edge list; the
ingested handle runs the same betweenness."""
import numpy as np
import pytest

import lgbc

pytestmark = pytest.mark.gpu


def _check(n, src, dst, directed):
    dev = lgbc.graph_from_edges(n, src, dst, directed=directed)
    cls = lgbc.SimpleDiGraph if directed else lgbc.SimpleGraph
    host = cls.from_edge_arrays(n, src, dst)
    rp, ci = dev.csr()
    hrp, hci = host.csr()
    assert np.array_equal(rp, hrp) and np.array_equal(ci, hci)
    if directed:
        irp, ici = dev.in_csr()
        hirp, hici = host.in_csr()
        assert np.array_equal(irp, hirp) and np.array_equal(ici, hici)
    return dev, host


@pytest.mark.parametrize("directed", [False, True])
def test_ingest_matches_host_storage(directed):
    rng = np.random.default_rng(3)
    n = 3000
    src = rng.integers(0, n, 40000)
    dst = rng.integers(0, n, 40000)
    src[:500] = dst[:500]  # self-loops
    src[500:1000], dst[500:1000] = src[1000:1500], dst[1000:1500]  # duplicates
    dev, host = _check(n, src, dst, directed)
    s = rng.choice(np.arange(1, n + 1), 200, replace=False)
    np.testing.assert_allclose(lgbc.betweenness_centrality(dev, s),
                               lgbc.betweenness_centrality(host, s), rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("directed", [False, True])
def test_ingest_edge_cases(directed):
    _check(5, np.zeros(0, np.int64), np.zeros(0, np.int64), directed)  # no edges
    g0 = lgbc.graph_from_edges(0, [], [], directed=directed)             # no vertices
    assert g0.nv() == 0 and len(g0.csr()[1]) == 0
    _check(1, [0], [0], directed)                                       # one self-loop
    _check(7, [6, 6, 0], [0, 0, 6], directed)                           # repeats both ways
    with pytest.raises((lgbc.ArgumentError, lgbc.BoundsError)):
        lgbc.graph_from_edges(3, [0, 3], [1, 1], directed=directed)


def test_ingest_large_power_of_two():
    # n = 2^18 exactly (the widest ids of the key width), 4M edges with repeats
    rng = np.random.default_rng(5)
    n = 1 << 18
    src = rng.integers(0, n, 1 << 22)
    dst = np.minimum(src + rng.geometric(0.001, 1 << 22), n - 1)
    g = lgbc.graph_from_edges(n, src, dst)
    rp, ci = g.csr()
    keys = np.unique(np.concatenate([src * n + dst, dst * n + src]))
    assert len(ci) == len(keys)
    assert np.array_equal(ci, (keys % n).astype(np.int32))
    assert np.array_equal(np.diff(rp), np.bincount(keys // n, minlength=n))
