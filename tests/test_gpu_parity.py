"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Bars: distances bit-exact; betweenness within 1e-9 relative per vertex with
zero compared to zero exactly (only the summation order differs from the
reference).  Every case runs on a real GPU.
"""
import numpy as np
import pytest

import lgbc
from lgbc import generators as G
from conftest import csr_args, make_graph
from oracle import oracle

pytestmark = pytest.mark.gpu

RTOL = 1e-9


def assert_bc_close(got, exp, rtol=RTOL):
    got = np.asarray(got)
    exp = np.asarray(exp)
    assert got.shape == exp.shape
    zero = exp == 0
    assert np.all(got[zero] == 0), np.nonzero(got[zero])[0][:10]
    nz = ~zero
    if np.any(nz):
        rel = np.abs(got[nz] - exp[nz]) / np.abs(exp[nz])
        assert rel.max() <= rtol, (rel.max(), np.argmax(rel))


def oracle_bc(g, sources0=None, normalize=True, endpoints=False, k=None, nthreads=4):
    rp, ci, kw = csr_args(g)
    src = np.arange(g.nv(), dtype=np.int32) if sources0 is None else np.asarray(sources0, np.int32)
    raw = oracle.betweenness_raw(rp, ci, src, endpoints=endpoints, nthreads=nthreads, **kw)
    return oracle.rescale(raw, g.nv(), normalize, g.is_directed(), len(src) if k is None else k)


def force_direction(g, mode):
    h = g.device_handle()
    if mode == "topdown":
        h.set_tuning(alpha=1e-12, beta=1e12)
    elif mode == "bottomup":
        h.set_tuning(alpha=1e12, beta=1e-12)
    else:
        h.set_tuning(alpha=14.0, beta=24.0)


# ---------------------------------------------------------------- known answers
def test_known_betweenness(known):
    for case in known["betweenness"]:
        g = make_graph(case)
        z = lgbc.betweenness_centrality(g, normalize=case["normalize"], endpoints=case["endpoints"])
        assert_bc_close(z, case["expected"])
    for case in known["betweenness_partial"]:
        g = make_graph(case)
        z = lgbc.betweenness_centrality(g, normalize=case["normalize"])
        for v in case["zero_at"]:
            assert z[v - 1] == 0.0


def test_golden_vector_float32(golden_graph, golden_bc, known):
    # test/centrality/betweenness.jl:8-17 on the GPU
    z = lgbc.betweenness_centrality(golden_graph)
    assert np.array_equal(z.astype(np.float32), golden_bc.astype(np.float32))
    assert_bc_close(z, golden_bc, rtol=1e-12)
    y = lgbc.betweenness_centrality(golden_graph, endpoints=True, normalize=False)
    assert np.array_equal(np.round(y[:3], 4), np.round(known["golden_endpoints"]["first3"], 4))
    # k-sampled and vs=1:20 (lengths, :21-25) plus value parity on the same sources
    x = lgbc.betweenness_centrality(golden_graph, 3, rng=0)
    assert len(x) == 50
    x2 = lgbc.betweenness_centrality(golden_graph, list(range(1, 21)))
    assert_bc_close(x2, oracle_bc(golden_graph, np.arange(20), k=20))


def test_parallel_names_equal_serial(golden_graph):
    z = lgbc.betweenness_centrality(golden_graph)
    for mode in ("threads", "distributed"):
        zp = lgbc.Parallel.betweenness_centrality(golden_graph, parallel=mode)
        assert np.array_equal(z, zp)


def test_gdistances_known(known):
    for entry in known["gdistances"]:
        g = make_graph(entry)
        for case in entry["cases"]:
            src = case["sources"]
            d = lgbc.gdistances(g, src if len(src) != 1 else src[0])
            exp = [np.iinfo(np.int64).max if x == "typemax" else x for x in case["expected"]]
            assert d.tolist() == exp
            assert lgbc.Parallel.gdistances(g, src).tolist() == exp
    # eltype typemax (bfs.jl:141, test/traversals/bfs.jl:33 with Int16 graphs)
    g16 = lgbc.SimpleGraph.from_edges(5, [(1, 2)], eltype=np.int16)
    d = lgbc.gdistances(g16, [])
    assert d.dtype == np.int16 and np.all(d == np.iinfo(np.int16).max)


# ---------------------------------------------------------------- random graphs
GRAPHS = {
    "er_undirected": lambda: G.erdos_renyi_nm(2000, 8000, seed=11),
    "er_directed": lambda: G.erdos_renyi_nm(2000, 8000, seed=12, directed=True),
    "rmat10": lambda: G.rmat(10, 16, seed=3),
    "rmat10_directed": lambda: G.rmat(10, 16, seed=4, directed=True),
    "ba": lambda: G.barabasi_albert(3000, 3, seed=5),
    "sparse_er": lambda: G.erdos_renyi_nm(3000, 2000, seed=6),  # many components
}


@pytest.mark.parametrize("name", sorted(GRAPHS))
@pytest.mark.parametrize("direction", ["auto", "topdown", "bottomup"])
def test_bc_exact_random(name, direction):
    g = GRAPHS[name]()
    force_direction(g, direction)
    z = lgbc.betweenness_centrality(g, normalize=False)
    assert_bc_close(z, oracle_bc(g, normalize=False))


@pytest.mark.parametrize("name", ["er_directed", "rmat10", "sparse_er"])
def test_bc_endpoints_and_sources(name):
    g = GRAPHS[name]()
    rng = np.random.default_rng(9)
    src = rng.choice(g.nv(), size=150, replace=True).astype(np.int32)  # duplicates allowed
    for endpoints in (False, True):
        for normalize in (False, True):
            z = lgbc.betweenness_centrality(g, list(src + 1), normalize=normalize, endpoints=endpoints)
            assert_bc_close(z, oracle_bc(g, src, normalize=normalize, endpoints=endpoints))


@pytest.mark.parametrize("lanes", [1, 7, 33, 64])
def test_lane_widths(lanes):
    g = GRAPHS["rmat10"]()
    g.device_handle().set_tuning(lanes=lanes)
    z = lgbc.betweenness_centrality(g, list(range(1, 200)), normalize=False)
    assert_bc_close(z, oracle_bc(g, np.arange(199), normalize=False))


@pytest.mark.parametrize("dense", [0, 2, 32])
@pytest.mark.parametrize("name", ["rmat10", "er_directed", "ba"])
def test_gather_paths(name, dense):
    # dense_edges selects, per 32-edge chunk, the edge-by-edge gather or the
    # bit-transposed one; both must give the oracle's result
    g = GRAPHS[name]()
    g.device_handle().set_tuning(dense_edges=dense, hub_degree=64)
    z = lgbc.betweenness_centrality(g, list(range(1, 300)), normalize=False)
    assert_bc_close(z, oracle_bc(g, np.arange(299), normalize=False))


@pytest.mark.parametrize("segment_degree", [0, 1000])
@pytest.mark.parametrize("name", ["rmat10", "er_directed", "ba", "sparse_er"])
def test_kernel_families(name, segment_degree):
    # segment_degree 0 forces the warp-per-vertex kernels, 1000 the
    # segmented (32 vertices per warp) kernels; both match the oracle
    g = GRAPHS[name]()
    g.device_handle().set_tuning(segment_degree=segment_degree, hub_degree=64)
    for ep in (False, True):
        z = lgbc.betweenness_centrality(g, list(range(1, 400)), normalize=False, endpoints=ep)
        assert_bc_close(z, oracle_bc(g, np.arange(399), normalize=False, endpoints=ep))


def test_sampled_k_uses_distinct_sources():
    g = GRAPHS["ba"]()
    rng = np.random.default_rng(123)
    z = lgbc.betweenness_centrality(g, 100, rng=rng)
    src = lgbc.sample(g.vertices(), 100, rng=np.random.default_rng(123))
    assert len(set(src)) == 100
    assert_bc_close(z, oracle_bc(g, np.asarray(src) - 1))


# ---------------------------------------------------------------- edge cases
def test_edge_cases():
    # empty graph, single vertex, no edges, isolated sources (degree 0 skipped)
    assert lgbc.betweenness_centrality(lgbc.SimpleGraph(0)).shape == (0,)
    assert lgbc.betweenness_centrality(lgbc.SimpleGraph(1)).tolist() == [0.0]
    g = lgbc.SimpleGraph(5)
    assert lgbc.betweenness_centrality(g).tolist() == [0.0] * 5
    assert lgbc.betweenness_centrality(g, endpoints=True).tolist() == [0.0] * 5
    assert lgbc.gdistances(g, 3).tolist() == [np.iinfo(np.int64).max] * 2 + [0] + \
        [np.iinfo(np.int64).max] * 2
    # digraph source with only in-arcs: degree > 0, reaches nothing, but counts
    # for endpoints (betweenness.jl:122)
    d = lgbc.SimpleDiGraph.from_edges(4, [(1, 2), (3, 2), (4, 2)])
    for ep in (False, True):
        z = lgbc.betweenness_centrality(d, [2, 1], normalize=False, endpoints=ep)
        assert_bc_close(z, oracle_bc(d, np.array([1, 0]), normalize=False, endpoints=ep))
    # complete graph, star
    kn = lgbc.SimpleGraph.from_edges(30, [(i, j) for i in range(1, 31) for j in range(i + 1, 31)])
    assert_bc_close(lgbc.betweenness_centrality(kn), oracle_bc(kn))
    star = lgbc.SimpleGraph.from_edges(500, [(1, j) for j in range(2, 501)])
    assert_bc_close(lgbc.betweenness_centrality(star), oracle_bc(star))


def test_long_path_grows_level_lists():
    # 64 sources spread along a 6000-vertex path: each vertex sits at many
    # distinct levels, so the level lists outgrow their first allocation
    n = 6000
    g = lgbc.SimpleGraph.from_edge_arrays(n, np.arange(n - 1), np.arange(1, n))
    src = np.linspace(0, n - 1, 64).astype(np.int32)
    z = lgbc.betweenness_centrality(g, list(src + 1), normalize=False)
    assert_bc_close(z, oracle_bc(g, src, normalize=False))
    d = lgbc.multi_gdistances(g, list(src + 1))
    rp, ci, _ = csr_args(g)
    for i in (0, 17, 63):
        assert np.array_equal(d[i], oracle.gdistances(rp, ci, [src[i]]).astype(g.eltype))


def test_grid_path_counts_overflow_replay():
    # test/centrality/betweenness.jl:74-77: path counts reach ~2.5e28 > 2^64,
    # so batches are replayed with FP64 path counts
    n1 = 50
    idx = lambda r, c: r * n1 + c
    e = np.asarray([(idx(r, c), idx(r, c + 1)) for r in range(n1) for c in range(n1 - 1)] +
                   [(idx(r, c), idx(r + 1, c)) for r in range(n1 - 1) for c in range(n1)])
    g = lgbc.SimpleGraph.from_edge_arrays(n1 * n1, e[:, 0], e[:, 1])
    z = lgbc.betweenness_centrality(g, normalize=False)
    assert z.max() < g.nv() * (g.nv() - 1)
    assert g.device_handle().stats()["wide_batches"] > 0
    assert_bc_close(z, oracle_bc(g, normalize=False, nthreads=8), rtol=1e-9)


# ---------------------------------------------------------------- gdistances
@pytest.mark.parametrize("name", sorted(GRAPHS))
@pytest.mark.parametrize("direction", ["auto", "topdown", "bottomup"])
def test_gdistances_random(name, direction):
    g = GRAPHS[name]()
    force_direction(g, direction)
    rp, ci, _ = csr_args(g)
    rng = np.random.default_rng(1)
    for srcs in ([0], [5, 17, 1000], rng.choice(g.nv(), 40).tolist()):
        got = lgbc.gdistances(g, [s + 1 for s in srcs])
        assert got.dtype == g.eltype
        exp = oracle.gdistances(rp, ci, srcs).astype(np.int64)
        exp[exp == oracle.UNREACHED32] = np.iinfo(g.eltype).max
        assert np.array_equal(got.astype(np.int64), exp)
    batch = rng.choice(g.nv(), 70).astype(np.int32)
    got = lgbc.multi_gdistances(g, list(batch + 1))
    for i, s in enumerate(batch):
        exp = oracle.gdistances(rp, ci, [s]).astype(np.int64)
        exp[exp == oracle.UNREACHED32] = np.iinfo(g.eltype).max
        assert np.array_equal(got[i].astype(np.int64), exp)


def test_gdistances_inplace_semantics():
    g = lgbc.SimpleGraph.from_edges(5, [(1, 2), (2, 3)])
    v = np.full(5, -7, np.int64)
    lgbc.gdistances_(g, 1, v)  # serial gdistances! leaves unreached entries alone
    assert v.tolist() == [0, 1, 2, -7, -7]
    lgbc.Parallel.gdistances_(g, [1], v)  # the Parallel one fills typemax first
    assert v.tolist() == [0, 1, 2] + [np.iinfo(np.int64).max] * 2


# ---------------------------------------------------------------- full size
def test_rmat20_properties():
    """Scale-20 R-MAT (the sampled-BC workload): GPU vs oracle on a source
    subset, and the dependency identity sum_v bc(v) = sum_s sum_t (d(s,t) - 1)
    checked between the Brandes and the distance kernels."""
    g = G.rmat(20, 16, seed=1)
    rp, ci, kw = csr_args(g)
    rng = np.random.default_rng(2)
    src = rng.choice(g.nv(), 64, replace=False).astype(np.int32)
    deg = np.diff(rp)
    act = src[deg[src] > 0]
    raw = lgbc.betweenness_raw(g, src)
    exp = oracle.betweenness_raw(rp, ci, src, nthreads=8, **kw)
    assert_bc_close(raw, exp)
    d = lgbc.multi_gdistances(g, list(act + 1)).astype(np.float64)
    d[d == np.iinfo(g.eltype).max] = np.nan
    ident = np.nansum(np.maximum(d - 1, 0))
    assert abs(raw.sum() - ident) <= 1e-9 * ident
    for s in act[:4]:
        got = lgbc.gdistances(g, int(s) + 1).astype(np.int64)
        e = oracle.gdistances(rp, ci, [s]).astype(np.int64)
        e[e == oracle.UNREACHED32] = np.iinfo(g.eltype).max
        assert np.array_equal(got, e)


# ---------------------------------------------------------------- many graphs
def test_betweenness_many_matches_per_graph():
    # uneven Barabasi-Albert graphs (plus a star, a path, an empty and an
    # edgeless graph) in one call; each graph against the oracle
    rng = np.random.default_rng(4)
    graphs = [G.barabasi_albert(int(n), 3, seed=1000 + i)
              for i, n in enumerate(rng.integers(20, 700, 40))]
    graphs += [lgbc.SimpleGraph.from_edges(70, [(1, j) for j in range(2, 71)]),
               lgbc.SimpleGraph.from_edge_arrays(300, np.arange(299), np.arange(1, 300)),
               lgbc.SimpleGraph(0), lgbc.SimpleGraph(5)]
    for endpoints in (False, True):
        res = lgbc.betweenness_centrality_many(graphs, normalize=False, endpoints=endpoints)
        assert len(res) == len(graphs)
        for g, z in zip(graphs, res):
            assert_bc_close(z, oracle_bc(g, normalize=False, endpoints=endpoints))
