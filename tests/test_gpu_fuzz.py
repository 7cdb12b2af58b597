"""Randomised cross-check: random graphs (sizes, densities, both kinds, hubs,
isolated vertices, self-loops) under random tunings -- lane width, hub cut,
gather strategy, direction thresholds, source ordering, device-driven loops,
stacked batches -- give the oracle's betweenness, stress and distances."""
import numpy as np
import pytest

import lgbc
from oracle import oracle

pytestmark = pytest.mark.gpu


def _graph(rng):
    n = int(rng.integers(2, 1500))
    m = int(rng.integers(0, 8 * n))
    directed = bool(rng.integers(0, 2))
    src = rng.integers(0, n, m)
    dst = rng.integers(0, n, m)
    if rng.random() < 0.5 and n > 10:  # a hub
        k = int(rng.integers(1, n))
        src = np.concatenate([src, np.zeros(k, np.int64)])
        dst = np.concatenate([dst, rng.integers(0, n, k)])
    cls = lgbc.SimpleDiGraph if directed else lgbc.SimpleGraph
    return cls.from_edge_arrays(n, src, dst)


def _tuning(rng):
    return dict(lanes=int(rng.choice([1, 7, 32, 48, 64, 65, 128])),
                hub_degree=int(rng.choice([2, 16, 256, 2**31 - 1])),
                dense_edges=int(rng.choice([0, 4, 32])),
                alpha=float(rng.choice([1.0, 14.0, 1e9])),
                beta=float(rng.choice([1.0, 24.0, 1e9])),
                source_order=int(rng.integers(0, 2)),
                graph_loop=int(rng.integers(0, 2)),
                stack_vertices=int(rng.choice([0, 1 << 21])),
                segment_degree=int(rng.choice([0, 1 << 30])),
                hub_order=int(rng.integers(0, 3)))


@pytest.mark.parametrize("seed", range(24))
def test_random_graphs_random_tunings(seed):
    rng = np.random.default_rng(1000 + seed)
    g = _graph(rng)
    h = g.device_handle()
    t = _tuning(rng)
    h.set_tuning(**t)
    rp, ci = g.csr()
    kw = {}
    if g.is_directed():
        irp, ici = g.in_csr()
        kw = dict(directed=True, in_rowptr=irp, in_colidx=ici)
    n = g.nv()
    k = int(rng.integers(1, min(n, 400) + 1))
    src = rng.choice(n, k, replace=bool(rng.integers(0, 2))).astype(np.int32)
    ends = bool(rng.integers(0, 2))
    got = lgbc.betweenness_centrality(g, src + 1, endpoints=ends)
    want = oracle.betweenness_centrality(rp, ci, src, endpoints=ends, **kw)
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9, err_msg=str(t))
    assert np.array_equal(lgbc.stress_centrality(g, src + 1), oracle.stress(rp, ci, src, **kw)), t
    d = lgbc.multi_gdistances(g, src[:70] + 1).astype(np.int64)
    for i, s in enumerate(src[:70].tolist()):
        od = oracle.gdistances(rp, ci, [s]).astype(np.int64)
        od[od == oracle.UNREACHED32] = np.iinfo(d.dtype).max if d.dtype != np.int64 else np.iinfo(np.int64).max
        dd = d[i].copy()
        assert np.array_equal(dd, od.astype(dd.dtype)), (t, s)


@pytest.mark.parametrize("seed", range(24, 56))
def test_random_graphs_random_tunings_more(seed):
    test_random_graphs_random_tunings(seed)


@pytest.mark.parametrize("seed", range(16))
def test_random_other_entry_points(seed):
    rng = np.random.default_rng(5000 + seed)
    g = _graph(rng)
    g.device_handle().set_tuning(**_tuning(rng))
    rp, ci = g.csr()
    kw = {}
    if g.is_directed():
        irp, ici = g.in_csr()
        kw = dict(directed=True, in_rowptr=irp, in_colidx=ici)
    n = g.nv()
    # weighted accumulation (repeats allowed)
    k = int(rng.integers(1, 300))
    src = rng.integers(0, n, k).astype(np.int32)
    w = rng.uniform(0.1, 4.0, k)
    _, want = oracle.dependency(rp, ci, src, w, **kw)
    got = lgbc.learned.betweenness_raw_weighted(g, src, w)
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9)
    # distance statistics -> closeness, eccentricity
    if n <= 600:
        assert np.array_equal(lgbc.closeness_centrality(g), oracle.closeness(rp, ci, g.degrees()))
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            assert np.array_equal(lgbc.eccentricity(g), oracle.eccentricity(rp, ci))
    # multi-source gdistances
    ms = rng.integers(0, n, int(rng.integers(0, 5))).astype(np.int32)
    d = lgbc.gdistances(g, ms + 1).astype(np.int64)
    od = oracle.gdistances(rp, ci, ms).astype(np.int64)
    od[od == oracle.UNREACHED32] = np.iinfo(np.int64).max
    assert np.array_equal(d, od)
    # BFS parents from a random vertex
    s = int(rng.integers(0, n))
    assert np.array_equal(lgbc.bfs_parents(g, s + 1).astype(np.int64),
                          oracle.bfs_parents(rp, ci, s) + 1)
    # core numbers (graphs without self-loops)
    if not np.any(ci == np.repeat(np.arange(n), np.diff(rp))):
        assert np.array_equal(lgbc.core_number(g), oracle.core_number(rp, ci, **kw))
    # device ingest of the same edges
    src0 = np.repeat(np.arange(n), np.diff(rp))
    dev = lgbc.graph_from_edges(n, src0, ci, directed=g.is_directed())
    assert np.array_equal(dev.csr()[1], ci) and np.array_equal(dev.csr()[0], rp)


@pytest.mark.parametrize("seed", range(6))
def test_random_many_graphs(seed):
    rng = np.random.default_rng(7000 + seed)
    graphs = []
    for _ in range(int(rng.integers(1, 12))):
        n = int(rng.integers(2, 400))
        m = int(rng.integers(0, 5 * n))
        graphs.append(lgbc.SimpleGraph.from_edge_arrays(n, rng.integers(0, n, m),
                                                        rng.integers(0, n, m)))
    ends = bool(rng.integers(0, 2))
    got = lgbc.betweenness_centrality_many(graphs, endpoints=ends)
    for g, b in zip(graphs, got):
        rp, ci = g.csr()
        np.testing.assert_allclose(b, oracle.betweenness_centrality(rp, ci, endpoints=ends),
                                   rtol=1e-9, atol=1e-9)
