"""Hub work item orders (tuning hub_order): every hub kernel
(top-down discovery, path-count pulls, dependency sweep, stress) reads the
items in that order and must give the oracle's results for every order,
sorted or unsorted rows, one or two lane words."""
import numpy as np
import pytest

import lgbc
from conftest import csr_args
from oracle import oracle
from test_gpu_parity import GRAPHS, assert_bc_close, force_direction, oracle_bc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("hub_order", [0, 1, 2])
@pytest.mark.parametrize("lanes", [64, 128])
@pytest.mark.parametrize("name", ["rmat10", "rmat10_directed", "ba"])
def test_orders_match_oracle(name, lanes, hub_order):
    g = GRAPHS[name]()
    g.device_handle().set_tuning(lanes=lanes, hub_degree=16, hub_order=hub_order,
                                 stack_vertices=0)
    rng = np.random.default_rng(hub_order + lanes)
    src = rng.choice(g.nv(), 200, replace=False).astype(np.int32)
    for ep in (False, True):
        z = lgbc.betweenness_centrality(g, list(src + 1), normalize=False, endpoints=ep)
        assert_bc_close(z, oracle_bc(g, src, normalize=False, endpoints=ep))
    rp, ci, kw = csr_args(g)
    assert np.array_equal(lgbc.stress_centrality(g, src[:90] + 1), oracle.stress(rp, ci, src[:90], **kw))


@pytest.mark.parametrize("direction", ["topdown", "bottomup"])
def test_orders_both_directions(direction):
    g = GRAPHS["rmat10"]()
    force_direction(g, direction)
    g.device_handle().set_tuning(hub_degree=8, hub_order=1)
    z = lgbc.betweenness_centrality(g, normalize=False)
    assert_bc_close(z, oracle_bc(g, normalize=False))


@pytest.mark.parametrize("hub_order", [1, 2])
def test_unsorted_rows(hub_order):
    # a CSR whose hub rows are not sorted by neighbour id: the item order is
    # then arbitrary, the result is unchanged
    g0 = GRAPHS["rmat10"]()
    rp, ci = g0.csr()
    rng = np.random.default_rng(2)
    ci2 = ci.copy()
    for v in range(len(rp) - 1):
        seg = ci2[rp[v]:rp[v + 1]]
        rng.shuffle(seg)
    g = lgbc.SimpleGraph.from_csr(rp, ci2.astype(np.int32), eltype=np.int32)
    g.device_handle().set_tuning(hub_degree=16, hub_order=hub_order)
    src = np.arange(0, 300, dtype=np.int32)
    z = lgbc.betweenness_centrality(g, list(src + 1), normalize=False)
    assert_bc_close(z, oracle_bc(g0, src, normalize=False))


def test_hub_order_validation():
    h = GRAPHS["ba"]().device_handle()
    with pytest.raises(Exception):
        h.set_tuning(hub_order=-1)
    with pytest.raises(Exception):
        h.set_tuning(hub_order=3)
    h.set_tuning(hub_order=0)
    assert h.tuning().hub_order == 0
