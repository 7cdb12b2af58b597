"""The autotuner (lgbc_tune): it leaves results unchanged, picks settings
from its candidate sets, and round-trips through its cache file."""
import numpy as np
import pytest

import lgbc
import lgbc.generators as gen

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("directed", [False, True])
def test_tune_keeps_results_and_uses_cache(tmp_path, directed):
    g = gen.rmat(13, 16, seed=31, directed=directed)
    src = np.arange(1, g.nv() + 1, 37)
    before = lgbc.betweenness_centrality(g, src)
    h = g.device_handle()
    cache = tmp_path / "tune.txt"
    chosen = h.tune(cache)
    assert chosen["hub_degree"] in (64, 128, 256, 512, 1024, 4096, 2**31 - 1)
    assert chosen["lanes"] in (32, 48, 64, 128)
    assert chosen["alpha"] in (2.0, 4.0, 8.0, 14.0, 24.0, 48.0)
    assert chosen["beta"] in (6.0, 12.0, 24.0, 48.0, 96.0)
    after = lgbc.betweenness_centrality(g, src)
    np.testing.assert_allclose(after, before, rtol=1e-9, atol=1e-12)
    line = cache.read_text().strip().splitlines()
    assert len(line) == 1 and line[0].startswith(f"n={g.nv()},nnz=")
    # a fresh handle takes the cached line without measuring
    h2 = lgbc.DeviceGraph(g)
    h2.set_tuning(hub_degree=99, lanes=5)
    assert h2.tune(cache) == chosen
    assert len(cache.read_text().strip().splitlines()) == 1
    h2.close()


def test_tune_graph_without_edges():
    g = lgbc.SimpleGraph.from_edges(10, [])
    h = g.device_handle()
    before = h.tuning()
    h.tune()
    assert h.tuning().lanes == before.lanes


@pytest.mark.parametrize("directed", [False, True])
def test_source_order_keeps_results(directed):
    g = gen.rmat(12, 16, seed=41, directed=directed)
    rng = np.random.default_rng(3)
    src = rng.choice(np.arange(1, g.nv() + 1), 700, replace=False)
    h = g.device_handle()
    h.set_tuning(source_order=0, lanes=64)
    a = lgbc.betweenness_centrality(g, src, endpoints=True)
    s0 = lgbc.stress_centrality(g, src)
    w = rng.uniform(0.5, 2.0, len(src))
    wa = lgbc.learned.betweenness_raw_weighted(g, (src - 1).astype(np.int32), w)
    h.set_tuning(source_order=1)
    b = lgbc.betweenness_centrality(g, src, endpoints=True)
    assert h.stats()["batches"] == (h.stats()["active_sources"] + 63) // 64
    np.testing.assert_allclose(b, a, rtol=1e-9, atol=1e-12)
    assert np.array_equal(lgbc.stress_centrality(g, src), s0)
    wb = lgbc.learned.betweenness_raw_weighted(g, (src - 1).astype(np.int32), w)
    np.testing.assert_allclose(wb, wa, rtol=1e-9, atol=1e-9)


def test_tuning_validation():
    g = gen.rmat(8, 4, seed=2)
    h = g.device_handle()
    for bad in (dict(source_order=2), dict(graph_loop=-1), dict(stack_vertices=-5),
                dict(lanes=0), dict(lanes=257), dict(alpha=0.0), dict(hub_degree=0)):
        with pytest.raises(lgbc.ArgumentError):
            h.set_tuning(**bad)
    h.set_tuning(lanes=7, source_order=0, graph_loop=0, stack_vertices=0)
    t = h.tuning()
    assert (t.lanes, t.source_order, t.graph_loop, t.stack_vertices) == (7, 0, 0, 0)
