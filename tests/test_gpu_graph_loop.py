"""Device-driven level loops (CUDA graphs with conditional nodes) give the
same results as the host-driven loops, through every path that uses them:
Brandes in both path-count kinds (with the FP64 replay), list growth,
distance batches, landmarks and the many-graph unions."""
import numpy as np
import pytest

import lgbc
import lgbc.generators as gen
from oracle import oracle

pytestmark = pytest.mark.gpu


def _both(g, fn):
    h = g.device_handle()
    out = []
    for mode in (0, 1):
        h.set_tuning(graph_loop=mode)
        out.append(fn())
    h.set_tuning(graph_loop=1)
    return out


@pytest.mark.parametrize("kind", ["rmat", "rmat_dir", "ba", "sparse"])
def test_betweenness_same_with_graph_loops(kind):
    rng = np.random.default_rng(11)
    if kind == "rmat":
        g = gen.rmat(13, 16, seed=5)
    elif kind == "rmat_dir":
        g = gen.rmat(13, 8, seed=6, directed=True)
    elif kind == "ba":
        g = gen.barabasi_albert(4000, 3, seed=7)
    else:
        e = rng.integers(1, 3001, size=(2500, 2))
        g = lgbc.SimpleGraph.from_edges(3000, [tuple(x) for x in e[e[:, 0] != e[:, 1]].tolist()])
    src = rng.choice(np.arange(1, g.nv() + 1), 300, replace=False)
    a, b = _both(g, lambda: lgbc.betweenness_centrality(g, src, endpoints=True))
    np.testing.assert_allclose(b, a, rtol=1e-12, atol=1e-15)
    rp, ci = g.csr()
    kw = {}
    if g.is_directed():
        irp, ici = g.in_csr()
        kw = dict(directed=True, in_rowptr=irp, in_colidx=ici)
    want = oracle.betweenness_centrality(rp, ci, (src - 1).astype(np.int32), endpoints=True, **kw)
    np.testing.assert_allclose(b, want, rtol=1e-9, atol=1e-12)
    d0, d1 = _both(g, lambda: lgbc.multi_gdistances(g, src[:70]))
    assert np.array_equal(d0, d1)


def test_wide_replay_and_list_growth_with_graph_loops():
    n = 50
    edges = [(r * n + c + 1, r * n + c + 2) for r in range(n) for c in range(n - 1)]
    edges += [(r * n + c + 1, (r + 1) * n + c + 1) for r in range(n - 1) for c in range(n)]
    grid = lgbc.SimpleGraph.from_edges(n * n, edges)
    a, b = _both(grid, lambda: lgbc.betweenness_centrality(grid, [1, 1250, 2500]))
    np.testing.assert_allclose(b, a, rtol=1e-12)
    assert grid.device_handle().stats()["wide_batches"] >= 1
    path = lgbc.SimpleGraph.from_edges(6000, [(i, i + 1) for i in range(1, 6000)])
    src = list(range(1, 6001, 97))
    a, b = _both(path, lambda: lgbc.betweenness_centrality(path, src))
    np.testing.assert_allclose(b, a, rtol=1e-12)
    rp, ci = path.csr()
    np.testing.assert_allclose(b, oracle.betweenness_centrality(rp, ci, np.array(src) - 1),
                               rtol=1e-9)


def test_many_graphs_with_graph_loops():
    graphs = [gen.barabasi_albert(int(n), 3, seed=50 + i) for i, n in enumerate([300, 450, 800, 1200])]
    h_default = [lgbc.betweenness_centrality_many(graphs)]
    for g, got in zip(graphs, h_default[0]):
        rp, ci = g.csr()
        np.testing.assert_allclose(got, oracle.betweenness_centrality(rp, ci), rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("directed,endpoints", [(False, False), (True, True)])
def test_stacked_batches_match(directed, endpoints):
    # 2000 vertices: 2^21 / 2000 copies allowed, so every batch of a call runs
    # in one stacked union; compare with stacking off and with the oracle
    g = gen.erdos_renyi_nm(2000, 7000, seed=9, directed=directed)
    rng = np.random.default_rng(4)
    src = rng.choice(np.arange(1, g.nv() + 1), 900, replace=False)
    h = g.device_handle()
    h.set_tuning(stack_vertices=0)
    a = lgbc.betweenness_centrality(g, src, endpoints=endpoints)
    h.set_tuning(stack_vertices=1 << 21)
    b = lgbc.betweenness_centrality(g, src, endpoints=endpoints)
    assert h.stats()["batches"] >= 1
    np.testing.assert_allclose(b, a, rtol=1e-9, atol=1e-12)
    rp, ci = g.csr()
    kw = {}
    if directed:
        irp, ici = g.in_csr()
        kw = dict(directed=True, in_rowptr=irp, in_colidx=ici)
    want = oracle.betweenness_centrality(rp, ci, (src - 1).astype(np.int32), endpoints=endpoints,
                                         **kw)
    np.testing.assert_allclose(b, want, rtol=1e-9, atol=1e-12)
    # all vertices, and a lane width that does not divide 64
    h.set_tuning(lanes=48)
    c = lgbc.betweenness_centrality(g)
    h.set_tuning(lanes=64, stack_vertices=0)
    d = lgbc.betweenness_centrality(g)
    np.testing.assert_allclose(c, d, rtol=1e-9, atol=1e-12)


def test_stacked_grid_replays_in_fp64():
    n = 40  # corner-to-corner path counts C(78, 39) > 2^64
    edges = [(r * n + c + 1, r * n + c + 2) for r in range(n) for c in range(n - 1)]
    edges += [(r * n + c + 1, (r + 1) * n + c + 1) for r in range(n - 1) for c in range(n)]
    g = lgbc.SimpleGraph.from_edges(n * n, edges)
    b = lgbc.betweenness_centrality(g)
    assert g.device_handle().stats()["wide_batches"] >= 1
    rp, ci = g.csr()
    np.testing.assert_allclose(b, oracle.betweenness_centrality(rp, ci), rtol=1e-9)


@pytest.mark.parametrize("directed", [False, True])
def test_weighted_batches_in_every_mode(directed):
    # importance weights through host-driven loops, device-driven loops and
    # stacked unions (one weight row per copy) give the same accumulation
    from lgbc.learned import betweenness_raw_weighted
    g = gen.erdos_renyi_nm(3000, 12000, seed=21, directed=directed)
    rng = np.random.default_rng(8)
    src = rng.integers(0, g.nv(), 700).astype(np.int32)
    w = rng.uniform(0.2, 3.0, len(src))
    h = g.device_handle()
    out = {}
    for loop in (0, 1):
        for stack in (0, 1 << 21):
            h.set_tuning(graph_loop=loop, stack_vertices=stack)
            out[(loop, stack)] = betweenness_raw_weighted(g, src, w)
    h.set_tuning(graph_loop=1, stack_vertices=1 << 21)
    base = out[(0, 0)]
    for key, val in out.items():
        np.testing.assert_allclose(val, base, rtol=1e-9, atol=1e-9, err_msg=str(key))
    rp, ci = g.csr()
    kw = {}
    if directed:
        irp, ici = g.in_csr()
        kw = dict(directed=True, in_rowptr=irp, in_colidx=ici)
    _, want = oracle.dependency(rp, ci, src, w, **kw)
    np.testing.assert_allclose(base, want, rtol=1e-9, atol=1e-9)


def test_stacked_batches_with_repeated_sources():
    # a source repeated inside one copy's batch becomes one seed with several lanes
    g = gen.erdos_renyi_nm(600, 1600, seed=13)
    rng = np.random.default_rng(6)
    src = rng.choice(np.arange(1, g.nv() + 1), 300, replace=True)
    src[:20] = src[0]
    h = g.device_handle()
    for lanes in (7, 64):
        h.set_tuning(lanes=lanes, stack_vertices=1 << 21)
        b = lgbc.betweenness_centrality(g, src)
        rp, ci = g.csr()
        want = oracle.betweenness_centrality(rp, ci, (src - 1).astype(np.int32))
        np.testing.assert_allclose(b, want, rtol=1e-9, atol=1e-12)
    h.set_tuning(lanes=64)
