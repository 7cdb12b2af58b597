"""Batches of 129-256 sources, which keep four 64-bit lane words per vertex:
top-down / bottom-up, hub items, both gather strategies, host- and
device-driven level loops, FP64 replay, weighted accumulation, stacked unions
and unions of graphs, against the oracle.  (The segmented low-degree kernels
exist for one and two words; four-word batches run the warp-per-vertex
kernels whatever segment_degree says.)"""
import numpy as np
import pytest

import lgbc
from lgbc import generators as G
from lgbc.learned import betweenness_raw_weighted
from conftest import csr_args
from oracle import oracle
from test_gpu_parity import GRAPHS, assert_bc_close, force_direction, oracle_bc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lanes", [129, 200, 256])
@pytest.mark.parametrize("name", ["rmat10", "er_directed", "ba", "rmat10_directed"])
def test_lane_widths_four_words(name, lanes):
    g = GRAPHS[name]()
    g.device_handle().set_tuning(lanes=lanes)
    src = np.arange(0, min(g.nv(), 600), dtype=np.int32)
    z = lgbc.betweenness_centrality(g, list(src + 1), normalize=False)
    assert_bc_close(z, oracle_bc(g, src, normalize=False))


@pytest.mark.parametrize("direction", ["auto", "topdown", "bottomup"])
@pytest.mark.parametrize("graph_loop", [0, 1])
@pytest.mark.parametrize("name", ["rmat10", "er_directed"])
def test_directions_and_loops_four_words(name, direction, graph_loop):
    g = GRAPHS[name]()
    force_direction(g, direction)
    g.device_handle().set_tuning(lanes=256, graph_loop=graph_loop)
    z = lgbc.betweenness_centrality(g, normalize=False)
    assert_bc_close(z, oracle_bc(g, normalize=False))


@pytest.mark.parametrize("dense", [0, 32])
@pytest.mark.parametrize("hub_degree", [4, 2**31 - 1])
@pytest.mark.parametrize("name", ["rmat10", "rmat10_directed"])
def test_gather_paths_and_hubs_four_words(name, hub_degree, dense):
    g = GRAPHS[name]()
    g.device_handle().set_tuning(lanes=256, hub_degree=hub_degree, dense_edges=dense,
                                 segment_degree=1000)
    rng = np.random.default_rng(hub_degree + dense)
    src = rng.choice(g.nv(), 520, replace=True).astype(np.int32)  # repeats allowed
    for ep in (False, True):
        z = lgbc.betweenness_centrality(g, list(src + 1), normalize=False, endpoints=ep)
        assert_bc_close(z, oracle_bc(g, src, normalize=False, endpoints=ep))


def test_dependency_df32_four_words():
    g = GRAPHS["rmat10"]()
    g.device_handle().set_tuning(lanes=256, dependency_df32=1)
    z = lgbc.betweenness_centrality(g, normalize=False)
    assert_bc_close(z, oracle_bc(g, normalize=False))


def test_overflow_replay_four_words():
    # 50 x 50 grid: path counts pass 2^64; 256-lane batches replay in FP64
    n1 = 50
    idx = lambda r, c: r * n1 + c
    e = np.asarray([(idx(r, c), idx(r, c + 1)) for r in range(n1) for c in range(n1 - 1)] +
                   [(idx(r, c), idx(r + 1, c)) for r in range(n1 - 1) for c in range(n1)])
    g = lgbc.SimpleGraph.from_edge_arrays(n1 * n1, e[:, 0], e[:, 1])
    g.device_handle().set_tuning(lanes=256, stack_vertices=0)
    src = np.arange(0, n1 * n1, 5, dtype=np.int32)
    z = lgbc.betweenness_centrality(g, list(src + 1), normalize=False)
    assert g.device_handle().stats()["wide_batches"] > 0
    assert_bc_close(z, oracle_bc(g, src, normalize=False, nthreads=8), rtol=1e-9)


def test_long_path_list_growth_four_words():
    # 256 sources along a path: every vertex sits at many distinct levels
    n = 6000
    g = lgbc.SimpleGraph.from_edge_arrays(n, np.arange(n - 1), np.arange(1, n))
    g.device_handle().set_tuning(lanes=256)
    src = np.linspace(0, n - 1, 256).astype(np.int32)
    z = lgbc.betweenness_centrality(g, list(src + 1), normalize=False)
    assert_bc_close(z, oracle_bc(g, src, normalize=False))


@pytest.mark.parametrize("name", ["rmat10", "er_directed"])
def test_weighted_four_words(name):
    g = GRAPHS[name]()
    g.device_handle().set_tuning(lanes=256, stack_vertices=0)
    rp, ci, kw = csr_args(g)
    rng = np.random.default_rng(4)
    src = rng.integers(0, g.nv(), size=500).astype(np.int32)
    w = rng.uniform(0.1, 5.0, size=500)
    got = betweenness_raw_weighted(g, src, w)
    _, want = oracle.dependency(rp, ci, src, w, **kw)
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9 * max(1.0, np.abs(want).max()))


def test_sampled_k_four_words_matches_two_words():
    g = GRAPHS["rmat10"]()
    g.device_handle().set_tuning(lanes=256)
    a = lgbc.betweenness_centrality(g, 600, rng=np.random.default_rng(5))
    g2 = GRAPHS["rmat10"]()
    g2.device_handle().set_tuning(lanes=128)
    b = lgbc.betweenness_centrality(g2, 600, rng=np.random.default_rng(5))
    assert_bc_close(a, b, rtol=1e-9)


@pytest.mark.parametrize("directed", [False, True])
def test_stacked_unions_four_words(directed):
    g = G.erdos_renyi_nm(1500, 6000, seed=22, directed=directed)
    h = g.device_handle()
    h.set_tuning(lanes=256, stack_vertices=1 << 21)
    rng = np.random.default_rng(9)
    src = rng.choice(g.nv(), 1300, replace=True).astype(np.int32)
    rp, ci, kw = csr_args(g)
    z = lgbc.betweenness_centrality(g, list(src + 1), normalize=False)
    assert_bc_close(z, oracle_bc(g, src, normalize=False))
    w = rng.uniform(0.1, 5.0, size=len(src))
    got = betweenness_raw_weighted(g, src, w)
    _, want = oracle.dependency(rp, ci, src, w, **kw)
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9 * max(1.0, np.abs(want).max()))


def test_tuning_limits_four_words():
    h = GRAPHS["ba"]().device_handle()
    h.set_tuning(lanes=256)
    assert h.tuning().lanes == 256
    with pytest.raises(Exception):
        h.set_tuning(lanes=257)
    assert h.tuning().lanes == 256
