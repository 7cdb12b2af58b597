"""GPU parity at the sizes of the benchmark configurations.

C1: the exact ER graph of the CPU-runnable configuration (n = 10,000,
    m = 50,000, seed 1, SimpleGraph{Int64}): betweenness_centrality(g;
    normalize=true, endpoints=false) over all 10^4 sources and gdistances(g, 1).
C3: Barabasi-Albert graphs spanning the configuration's n in [200, 20,000]
    (k = 3) in one lgbc_betweenness_many call, each graph exact.
C4: the directed R-MAT scale-22 graph (16 n arc draws, seed 1) on a 64-source
    subset: the 64-lane batch with direction switching on the in/out CSR, and
    once more with every level forced bottom-up (the lane-filtered kernels).
Bars: distances bit-exact, betweenness within 1e-9 relative per vertex with 0
compared to 0 exactly.  The oracle runs multi-threaded (fast BFS mode, the
same values as its heap mode).
"""
import os

import numpy as np
import pytest

import lgbc
from lgbc import generators as G
from conftest import csr_args
from oracle import oracle
from test_gpu_parity import assert_bc_close, oracle_bc

pytestmark = pytest.mark.gpu

NT = max(1, min(16, os.cpu_count() or 1))


def test_c1_er10k_exact_size():
    g = G.erdos_renyi_nm(10000, 50000, seed=1, eltype=np.int64)
    assert g.nv() == 10000 and g.ne() == 50000 and g.eltype == np.int64
    z = lgbc.betweenness_centrality(g, normalize=True, endpoints=False)
    assert_bc_close(z, oracle_bc(g, normalize=True, nthreads=NT))
    rp, ci, _ = csr_args(g)
    d = lgbc.gdistances(g, 1)
    e = oracle.gdistances(rp, ci, [0]).astype(np.int64)
    e[e == oracle.UNREACHED32] = np.iinfo(np.int64).max
    assert d.dtype == np.int64 and np.array_equal(d, e)
    # the df32 opt-in meets the same bar on this graph
    h = g.device_handle()
    h.set_tuning(dependency_df32=1)
    try:
        z2 = lgbc.betweenness_centrality(g, normalize=True, endpoints=False)
    finally:
        h.set_tuning(dependency_df32=0)
    assert_bc_close(z2, z)


def test_c3_ba_graphs_up_to_20000():
    ns = [200, 201, 1500, 4096, 9000, 14000, 20000, 20000]
    graphs = [G.barabasi_albert(n, 3, seed=1000 + i) for i, n in enumerate(ns)]
    for g, n in zip(graphs, ns):
        assert g.nv() == n and g.ne() == 3 * (n - 3)
    res = lgbc.betweenness_centrality_many(graphs, normalize=False)
    for g, z in zip(graphs, res):
        assert_bc_close(z, oracle_bc(g, normalize=False, nthreads=NT))


@pytest.fixture(scope="module")
def rmat22_directed():
    return G.rmat(22, 16, seed=1, directed=True)


@pytest.mark.parametrize("direction", ["auto", "bottomup"])
def test_c4_rmat22_directed_subset(rmat22_directed, direction):
    g = rmat22_directed
    assert g.is_directed() and g.nv() == 1 << 22
    rp, ci, kw = csr_args(g)
    rng = np.random.default_rng(5)
    deg = g.degrees()
    src = rng.choice(np.flatnonzero(deg > 0), 64, replace=False).astype(np.int32)
    h = g.device_handle()
    if direction == "bottomup":
        h.set_tuning(alpha=1e12, beta=1e-12)
    try:
        raw = lgbc.betweenness_raw(g, src)
        st = h.stats()
    finally:
        h.set_tuning(alpha=14.0, beta=24.0)
    assert st["bottomup_levels"] > 0
    exp = oracle.betweenness_raw(rp, ci, src, nthreads=NT, **kw)
    assert_bc_close(raw, exp)
    if direction == "auto":
        for s in src[:3]:
            got = lgbc.gdistances(g, int(s) + 1).astype(np.int64)
            e = oracle.gdistances(rp, ci, [s]).astype(np.int64)
            e[e == oracle.UNREACHED32] = np.iinfo(g.eltype).max
            assert np.array_equal(got, e)
