"""Pin the CPU oracle to the reference's own golden vectors and known answers.

Every expected value here comes from LightGraphs.jl v1.3.5's tests, copied into
tests/golden/ by tests/golden/make_golden.py.  No GPU needed.
"""
import numpy as np
import pytest

from conftest import csr_args, make_graph

from oracle import oracle


@pytest.mark.parametrize("mode", ["faithful", "fast"])
def test_golden_bc_float32_equal(golden_graph, golden_bc, mode):
    # test/centrality/betweenness.jl:8-13: map(Float32, z) == map(Float32, c)
    rp, ci, kw = csr_args(golden_graph)
    assert golden_graph.is_directed() and golden_graph.nv() == 50 and golden_graph.ne() == 500
    z = oracle.betweenness_centrality(rp, ci, mode=mode, **kw)
    assert np.array_equal(z.astype(np.float32), golden_bc.astype(np.float32))
    assert np.max(np.abs(z - golden_bc) / np.abs(golden_bc)) < 1e-12


@pytest.mark.parametrize("mode", ["faithful", "fast"])
def test_golden_endpoints_triple(golden_graph, known, mode):
    # test/centrality/betweenness.jl:15-17
    case = known["golden_endpoints"]
    rp, ci, kw = csr_args(golden_graph)
    y = oracle.betweenness_centrality(rp, ci, normalize=False, endpoints=True, mode=mode, **kw)
    assert np.array_equal(np.round(y[:3], 4), np.round(case["first3"], 4))


@pytest.mark.parametrize("mode", ["faithful", "fast"])
def test_known_betweenness(known, mode):
    for case in known["betweenness"]:
        g = make_graph(case)
        rp, ci, kw = csr_args(g)
        z = oracle.betweenness_centrality(rp, ci, normalize=case["normalize"],
                                          endpoints=case["endpoints"], mode=mode, **kw)
        assert np.array_equal(z, np.asarray(case["expected"])), case["name"]


def test_known_partial(known):
    for case in known["betweenness_partial"]:
        g = make_graph(case)
        rp, ci, kw = csr_args(g)
        z = oracle.betweenness_centrality(rp, ci, normalize=case["normalize"], **kw)
        for v in case["zero_at"]:
            assert z[v - 1] == 0.0


def test_two_vertex_sources_forms_agree():
    # test/centrality/betweenness.jl:31-37: default vs range vs vector
    rp = np.array([0, 1, 2]); ci = np.array([1, 0], np.int32)
    a = oracle.betweenness_centrality(rp, ci)
    b = oracle.betweenness_centrality(rp, ci, sources=np.arange(2))
    assert np.array_equal(a, b) and np.all(a == 0)


def test_dijkstra_state(known):
    # test/shortestpaths/dijkstra.jl:77-103
    c0, c1 = known["dijkstra"]
    g = make_graph(c0)
    rp, ci, _ = csr_args(g)
    d, pc, preds, closest = oracle.dijkstra(rp, ci, c0["source"] - 1)
    assert pc.tolist() == c0["pathcounts"]
    assert [[u + 1 for u in p] for p in preds] == c0["predecessors"]
    assert (closest + 1).tolist() == c0["closest_vertices"]
    g = make_graph(c1)
    rp, ci, _ = csr_args(g)
    _, _, _, closest = oracle.dijkstra(rp, ci, c1["source"] - 1)
    assert (closest + 1).tolist() == c1["closest_vertices"]


def test_gdistances_known(known):
    # test/traversals/bfs.jl:29-35, test/parallel/traversals/gdistances.jl:4-18
    for entry in known["gdistances"]:
        g = make_graph(entry)
        rp, ci, _ = csr_args(g)
        for case in entry["cases"]:
            d = oracle.gdistances(rp, ci, np.asarray(case["sources"], np.int32) - 1)
            exp = [oracle.UNREACHED32 if x == "typemax" else x for x in case["expected"]]
            assert d.tolist() == exp


def test_parallel_equals_serial(golden_graph):
    # test/parallel/centrality/betweenness.jl:8-22: threaded == serial (isapprox)
    rp, ci, kw = csr_args(golden_graph)
    z = oracle.betweenness_centrality(rp, ci, mode="faithful", **kw)
    for nt in (2, 4):
        zt = oracle.betweenness_centrality(rp, ci, mode="faithful", nthreads=nt, **kw)
        assert np.allclose(z, zt, rtol=1e-12, atol=0)
        y = oracle.betweenness_centrality(rp, ci, normalize=False, endpoints=True,
                                          mode="fast", nthreads=nt, **kw)
        y1 = oracle.betweenness_centrality(rp, ci, normalize=False, endpoints=True,
                                           mode="faithful", **kw)
        assert np.allclose(y, y1, rtol=1e-12, atol=0)


def test_grid_path_counts_above_2_53():
    # test/centrality/betweenness.jl:74-77: grid([50, 50]), normalize=false
    import lgbc
    n1 = 50
    idx = lambda r, c: r * n1 + c
    e = [(idx(r, c), idx(r, c + 1)) for r in range(n1) for c in range(n1 - 1)] + \
        [(idx(r, c), idx(r + 1, c)) for r in range(n1 - 1) for c in range(n1)]
    e = np.asarray(e)
    g = lgbc.SimpleGraph.from_edge_arrays(n1 * n1, e[:, 0], e[:, 1])
    rp, ci, _ = csr_args(g)
    z = oracle.betweenness_centrality(rp, ci, normalize=False, nthreads=4)
    assert z.max() < g.nv() * (g.nv() - 1)


def test_networkx_cross_check():
    # independent check of the oracle against networkx (unnormalised, halved
    # for undirected graphs exactly like _rescale! with normalize=false)
    nx = pytest.importorskip("networkx")
    import lgbc
    from lgbc import generators as G
    for directed in (False, True):
        g = G.erdos_renyi_nm(300, 900, seed=7, directed=directed)
        rp, ci, kw = csr_args(g)
        z = oracle.betweenness_centrality(rp, ci, normalize=False, **kw)
        H = nx.DiGraph() if directed else nx.Graph()
        H.add_nodes_from(range(g.nv()))
        src = np.repeat(np.arange(g.nv()), np.diff(rp))
        H.add_edges_from(zip(src.tolist(), ci.tolist()))
        ref = nx.betweenness_centrality(H, normalized=False)
        r = np.array([ref[v] for v in range(g.nv())])
        assert np.allclose(z, r, rtol=1e-10, atol=1e-9)


@pytest.mark.parametrize("directed", [False, True])
def test_faithful_equals_fast_on_random(directed):
    from lgbc import generators as G
    g = G.erdos_renyi_nm(500, 2000, seed=3, directed=directed)
    rp, ci, kw = csr_args(g)
    src = np.arange(0, 500, 7, dtype=np.int32)
    for ep in (False, True):
        a = oracle.betweenness_raw(rp, ci, src, endpoints=ep, mode="faithful", **kw)
        b = oracle.betweenness_raw(rp, ci, src, endpoints=ep, mode="fast", nthreads=3, **kw)
        assert np.allclose(a, b, rtol=1e-12, atol=1e-12)
