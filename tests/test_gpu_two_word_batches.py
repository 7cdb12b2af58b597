"""Batches of 65-128 sources, which keep two 64-bit lane words per vertex:
every kernel family (top-down / bottom-up, hub items, both gather strategies,
segmented warps, host- and device-driven level loops, FP64 replay, weighted
accumulation, stacked unions and unions of graphs) against the oracle, and
the entry points that stay at 64 lanes with such a tuning set."""
import numpy as np
import pytest

import lgbc
from lgbc import generators as G
from lgbc.learned import betweenness_raw_weighted
from conftest import csr_args
from oracle import oracle
from test_gpu_parity import GRAPHS, assert_bc_close, force_direction, oracle_bc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lanes", [65, 100, 128])
@pytest.mark.parametrize("name", ["rmat10", "er_directed", "ba", "rmat10_directed"])
def test_lane_widths_two_words(name, lanes):
    g = GRAPHS[name]()
    g.device_handle().set_tuning(lanes=lanes)
    src = np.arange(0, min(g.nv(), 300), dtype=np.int32)
    z = lgbc.betweenness_centrality(g, list(src + 1), normalize=False)
    assert_bc_close(z, oracle_bc(g, src, normalize=False))


@pytest.mark.parametrize("direction", ["auto", "topdown", "bottomup"])
@pytest.mark.parametrize("graph_loop", [0, 1])
@pytest.mark.parametrize("name", ["rmat10", "er_directed", "sparse_er"])
def test_directions_and_loops(name, direction, graph_loop):
    g = GRAPHS[name]()
    force_direction(g, direction)
    g.device_handle().set_tuning(lanes=128, graph_loop=graph_loop)
    z = lgbc.betweenness_centrality(g, normalize=False)
    assert_bc_close(z, oracle_bc(g, normalize=False))


@pytest.mark.parametrize("dense", [0, 2, 32])
@pytest.mark.parametrize("hub_degree", [4, 64, 2**31 - 1])
@pytest.mark.parametrize("name", ["rmat10", "rmat10_directed", "ba"])
def test_gather_paths_and_hubs(name, hub_degree, dense):
    g = GRAPHS[name]()
    g.device_handle().set_tuning(lanes=128, hub_degree=hub_degree, dense_edges=dense)
    rng = np.random.default_rng(hub_degree + dense)
    src = rng.choice(g.nv(), 260, replace=True).astype(np.int32)  # repeats allowed
    for ep in (False, True):
        z = lgbc.betweenness_centrality(g, list(src + 1), normalize=False, endpoints=ep)
        assert_bc_close(z, oracle_bc(g, src, normalize=False, endpoints=ep))


@pytest.mark.parametrize("name", ["rmat10", "er_directed", "ba", "sparse_er"])
def test_segmented_kernels(name):
    g = GRAPHS[name]()
    g.device_handle().set_tuning(lanes=128, segment_degree=1000, hub_degree=64)
    z = lgbc.betweenness_centrality(g, list(range(1, 400)), normalize=False)
    assert_bc_close(z, oracle_bc(g, np.arange(399), normalize=False))


def test_sampled_k_two_words():
    g = GRAPHS["rmat10"]()
    g.device_handle().set_tuning(lanes=128)
    a = lgbc.betweenness_centrality(g, 300, rng=np.random.default_rng(5))
    g2 = GRAPHS["rmat10"]()
    g2.device_handle().set_tuning(lanes=64)
    b = lgbc.betweenness_centrality(g2, 300, rng=np.random.default_rng(5))
    assert_bc_close(a, b, rtol=1e-9)


def test_overflow_replay_two_words():
    # 50 x 50 grid: path counts pass 2^64; 128-lane batches replay in FP64
    n1 = 50
    idx = lambda r, c: r * n1 + c
    e = np.asarray([(idx(r, c), idx(r, c + 1)) for r in range(n1) for c in range(n1 - 1)] +
                   [(idx(r, c), idx(r + 1, c)) for r in range(n1 - 1) for c in range(n1)])
    g = lgbc.SimpleGraph.from_edge_arrays(n1 * n1, e[:, 0], e[:, 1])
    g.device_handle().set_tuning(lanes=128, stack_vertices=0)
    src = np.arange(0, n1 * n1, 9, dtype=np.int32)
    z = lgbc.betweenness_centrality(g, list(src + 1), normalize=False)
    assert g.device_handle().stats()["wide_batches"] > 0
    assert_bc_close(z, oracle_bc(g, src, normalize=False, nthreads=8), rtol=1e-9)


def test_long_path_list_growth_two_words():
    # 128 sources along a path: every vertex sits at many distinct levels
    n = 6000
    g = lgbc.SimpleGraph.from_edge_arrays(n, np.arange(n - 1), np.arange(1, n))
    g.device_handle().set_tuning(lanes=128)
    src = np.linspace(0, n - 1, 128).astype(np.int32)
    z = lgbc.betweenness_centrality(g, list(src + 1), normalize=False)
    assert_bc_close(z, oracle_bc(g, src, normalize=False))


@pytest.mark.parametrize("name", ["rmat10", "er_directed"])
def test_weighted_two_words(name):
    g = GRAPHS[name]()
    g.device_handle().set_tuning(lanes=128, stack_vertices=0)
    rp, ci, kw = csr_args(g)
    rng = np.random.default_rng(3)
    src = rng.integers(0, g.nv(), size=250).astype(np.int32)
    w = rng.uniform(0.1, 5.0, size=250)
    got = betweenness_raw_weighted(g, src, w)
    _, want = oracle.dependency(rp, ci, src, w, **kw)
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9 * max(1.0, np.abs(want).max()))


def test_other_entry_points_with_wide_tuning():
    # stress and distance batches run at most 64 lanes whatever the tuning
    g = GRAPHS["rmat10"]()
    g.device_handle().set_tuning(lanes=128)
    rp, ci, _ = csr_args(g)
    src = np.arange(0, 150, dtype=np.int32)
    assert np.array_equal(lgbc.stress_centrality(g, src + 1), oracle.stress(rp, ci, src))
    d = lgbc.multi_gdistances(g, src + 1).astype(np.int64)
    for i in (0, 77, 149):
        assert np.array_equal(d[i], oracle.gdistances(rp, ci, [src[i]]).astype(np.int64))


def test_tuning_limits():
    h = GRAPHS["ba"]().device_handle()
    h.set_tuning(lanes=128)
    assert h.tuning().lanes == 128
    with pytest.raises(Exception):
        h.set_tuning(lanes=0)
    assert h.tuning().lanes == 128


@pytest.mark.parametrize("directed", [False, True])
def test_stacked_unions_two_words(directed):
    # a small graph runs as a stacked union of copies, each holding a 128-lane
    # batch; repeated sources inside one copy share a seed
    g = G.erdos_renyi_nm(1500, 6000, seed=21, directed=directed)
    h = g.device_handle()
    h.set_tuning(lanes=128, stack_vertices=1 << 21)
    rng = np.random.default_rng(8)
    src = rng.choice(g.nv(), 700, replace=True).astype(np.int32)
    rp, ci, kw = csr_args(g)
    for ep in (False, True):
        z = lgbc.betweenness_centrality(g, list(src + 1), normalize=False, endpoints=ep)
        assert_bc_close(z, oracle_bc(g, src, normalize=False, endpoints=ep))
    w = rng.uniform(0.1, 5.0, size=len(src))
    got = betweenness_raw_weighted(g, src, w)
    _, want = oracle.dependency(rp, ci, src, w, **kw)
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9 * max(1.0, np.abs(want).max()))


def test_many_graphs_two_words():
    # unions of graphs run 128 lanes per batch by default
    gs = [G.barabasi_albert(int(n), 3, seed=50 + i) for i, n in enumerate([90, 300, 1200, 700, 130])]
    gs.append(G.erdos_renyi_nm(400, 900, seed=5))
    outs = lgbc.betweenness_centrality_many(gs, normalize=False)
    for g, z in zip(gs, outs):
        assert_bc_close(z, oracle_bc(g, normalize=False))


@pytest.mark.parametrize("endpoints", [False, True])
def test_many_graphs_two_groups_in_flight(endpoints):
    # a 2,097,000-vertex graph (a 600-vertex BA component, the rest isolated)
    # fills one union group alone, so the small graphs form a second group,
    # run at the same time from a second host thread
    small = G.barabasi_albert(600, 3, seed=77)
    rp, ci = small.csr()
    n_big = 2_097_000
    big = lgbc.SimpleGraph.from_csr(np.concatenate([rp, np.full(n_big - small.nv(), rp[-1])]), ci)
    gs = [G.barabasi_albert(int(n), 3, seed=90 + i) for i, n in enumerate([500, 140, 800])]
    outs = lgbc.betweenness_centrality_many([big] + gs, normalize=False, endpoints=endpoints)
    # with endpoints, each source of degree > 0 (isolated ones are skipped)
    # adds n - 1 to itself and 1 to every other vertex, reached or not
    # (_accumulate_endpoints! walks all n vertices): after the undirected
    # halving, + (n_big - 600) / 2 on the component and 600 / 2 on each
    # isolated vertex
    extra = (n_big - small.nv()) / 2 if endpoints else 0.0
    assert_bc_close(outs[0][:small.nv()],
                    oracle_bc(small, normalize=False, endpoints=endpoints) + extra)
    assert np.all(outs[0][small.nv():] == (small.nv() / 2 if endpoints else 0.0))
    for g, z in zip(gs, outs[1:]):
        assert_bc_close(z, oracle_bc(g, normalize=False, endpoints=endpoints))
