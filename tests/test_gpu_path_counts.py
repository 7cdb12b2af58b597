"""GPU parity of the path counts: lgbc_path_counts against the oracle.

dijkstra_shortest_paths(g, s) with unit weights keeps pathcounts (sigma) as
Float64 sums (src/shortestpaths/dijkstra.jl:102,118) and its dists; the GPU
keeps sigma as exact uint64 integers.  Where the counts stay below 2^53 the
reference's Float64 sums are exact too, so the two must agree bit for bit;
above 2^64 the GPU recomputes the batch with FP64 counts, whose value depends
on the summation order (as the reference's does on its heap order), so those
cases are compared to a relative 1e-12.
"""
import math

import numpy as np
import pytest

import lgbc
from lgbc import generators as G
from conftest import csr_args, make_graph
from oracle import oracle
from test_gpu_parity import GRAPHS

pytestmark = pytest.mark.gpu

I64MAX = np.iinfo(np.int64).max


def oracle_row(g, s0):
    rp, ci, _ = csr_args(g)
    d, pc, _, _ = oracle.dijkstra(rp, ci, int(s0))
    return pc, d


def test_dijkstra_fixture(known):
    # test/shortestpaths/dijkstra.jl:77-93: pathcounts [1, 1, 1, 1, 2] from vertex 1
    for case in known["dijkstra"]:
        g = make_graph(case)
        pc, d = lgbc.path_counts(g, [case["source"]])
        exp_pc, exp_d = oracle_row(g, case["source"] - 1)
        assert np.array_equal(pc[0], exp_pc)
        assert np.array_equal(d[0].astype(np.int64), exp_d)
        if "pathcounts" in case:
            assert pc[0].tolist() == case["pathcounts"]


@pytest.mark.parametrize("name", sorted(GRAPHS))
def test_path_counts_bit_exact(name):
    g = GRAPHS[name]()
    rng = np.random.default_rng(7)
    # 70 sources: two batches, a repeated source, vertex 1 and a random tail
    src0 = np.concatenate([[0, 0], rng.choice(g.nv(), 68)]).astype(np.int32)
    pc, d = lgbc.path_counts(g, list(src0 + 1))
    assert pc.shape == (70, g.nv()) and d.dtype == g.eltype
    for i in (0, 1, 2, 35, 64, 69):
        exp_pc, exp_d = oracle_row(g, src0[i])
        assert exp_pc.max() < 2.0**53
        assert np.array_equal(pc[i], exp_pc), i
        exp_d = exp_d.copy()
        exp_d[exp_d == I64MAX] = np.iinfo(g.eltype).max
        assert np.array_equal(d[i].astype(np.int64), exp_d), i


def test_path_counts_directions_agree():
    # the same counts whichever BFS direction each level takes
    g = GRAPHS["rmat10_directed"]()
    src = list(range(1, 65))
    ref, _ = lgbc.path_counts(g, src)
    h = g.device_handle()
    try:
        for a, b in ((1e-12, 1e12), (1e12, 1e-12)):
            h.set_tuning(alpha=a, beta=b)
            got, _ = lgbc.path_counts(g, src)
            assert np.array_equal(got, ref)
    finally:
        h.set_tuning(alpha=14.0, beta=24.0)


def test_path_counts_past_2_64():
    # the 50 x 50 grid of test/centrality/betweenness.jl:74-77: counts reach
    # C(98, 49) ~ 2.5e28 > 2^64, so the batch is recomputed with FP64 counts
    n1 = 50
    idx = lambda r, c: r * n1 + c
    e = np.asarray([(idx(r, c), idx(r, c + 1)) for r in range(n1) for c in range(n1 - 1)] +
                   [(idx(r, c), idx(r + 1, c)) for r in range(n1 - 1) for c in range(n1)])
    g = lgbc.SimpleGraph.from_edge_arrays(n1 * n1, e[:, 0], e[:, 1])
    pc, d = lgbc.path_counts(g, [1, 1250])
    assert g.device_handle().stats()["wide_batches"] > 0
    for i, s0 in enumerate((0, 1249)):
        exp_pc, exp_d = oracle_row(g, s0)
        small = exp_pc < 2.0**53
        assert np.array_equal(pc[i][small], exp_pc[small])
        assert np.allclose(pc[i][~small], exp_pc[~small], rtol=1e-12, atol=0)
        assert np.array_equal(d[i].astype(np.int64), exp_d)
    # the corner-to-corner count is the binomial coefficient
    assert pc[0][idx(49, 49)] == pytest.approx(float(math.comb(98, 49)), rel=1e-15)


def test_path_counts_rmat20():
    # the default bench graph: two sources against the oracle, and for all
    # eight the defining recursion sigma[v] = sum of sigma over in-neighbours
    # one level closer, checked on every edge at once
    g = G.rmat(20, 16, seed=1)
    rng = np.random.default_rng(3)
    deg = g.degrees()
    src0 = rng.choice(np.flatnonzero(deg > 0), 8, replace=False).astype(np.int32)
    pc, d = lgbc.path_counts(g, list(src0 + 1))
    for i in (0, 5):
        exp_pc, exp_d = oracle_row(g, src0[i])
        small = exp_pc < 2.0**53
        assert np.array_equal(pc[i][small], exp_pc[small])
        assert np.allclose(pc[i][~small], exp_pc[~small], rtol=1e-12, atol=0)
        exp_d = exp_d.copy()
        exp_d[exp_d == I64MAX] = np.iinfo(g.eltype).max
        assert np.array_equal(d[i].astype(np.int64), exp_d)
    rp, ci = g.csr()
    u = np.repeat(np.arange(g.nv()), np.diff(rp))  # edge u -> ci (undirected: both ways)
    for i in range(8):
        di = d[i].astype(np.int64)
        reach = di != np.iinfo(g.eltype).max
        dag = reach[u] & reach[ci] & (di[ci] == di[u] + 1)
        s = np.zeros(g.nv())
        np.add.at(s, ci[dag], pc[i][u[dag]])
        s[src0[i]] = 1.0
        assert np.allclose(pc[i][reach], s[reach], rtol=1e-13, atol=0)
        assert np.all(pc[i][~reach] == 0)
