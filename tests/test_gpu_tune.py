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
    assert chosen["lanes"] in (32, 48, 64)
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
