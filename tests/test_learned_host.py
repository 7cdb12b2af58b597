"""CPU checks of the learned-proposal pieces: the oracle's core numbers,
dependency masses and FP64 MLP are pinned against independent computations,
and the host-side estimator helpers are exercised without a GPU."""
import numpy as np
import pytest

import lgbc
from lgbc import _lib
from lgbc.learned import l1_error, top_rank_error
from oracle import mlp as omlp
from oracle import oracle


def _random_graph(n, m, seed, directed=False):
    rng = np.random.default_rng(seed)
    edges = set()
    while len(edges) < m:
        u, v = rng.integers(1, n + 1, size=2)
        if u == v:
            continue
        edges.add((int(u), int(v)) if directed else (int(min(u, v)), int(max(u, v))))
    cls = lgbc.SimpleDiGraph if directed else lgbc.SimpleGraph
    return cls.from_edges(n, sorted(edges))


def test_core_number_doc_example():
    # src/degeneracy.jl:25-36: path_graph(5), add_vertex!, add_edge!(g, 5, 2)
    g = lgbc.SimpleGraph.from_edges(6, [(1, 2), (2, 3), (3, 4), (4, 5), (5, 2)])
    rp, ci = g.csr()
    assert oracle.core_number(rp, ci).tolist() == [1, 2, 2, 2, 2, 0]


def test_core_number_rejects_self_loops():
    g = lgbc.SimpleGraph.from_edges(3, [(1, 1), (1, 2)])
    rp, ci = g.csr()
    with pytest.raises(ValueError):
        oracle.core_number(rp, ci)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_core_number_matches_networkx(seed):
    nx = pytest.importorskip("networkx")
    g = _random_graph(300, 900 + 300 * seed, seed)
    rp, ci = g.csr()
    G = nx.Graph()
    G.add_nodes_from(range(300))
    for v in range(300):
        for u in ci[rp[v]:rp[v + 1]]:
            G.add_edge(v, int(u))
    want = nx.core_number(G)
    assert oracle.core_number(rp, ci).tolist() == [want[v] for v in range(300)]


@pytest.mark.parametrize("seed", [4, 5])
def test_directed_core_number_matches_networkx(seed):
    # digraph: degree = out + in, reciprocal arcs count twice (src/degeneracy.jl:41,91-96);
    # networkx defines directed core numbers with the same in + out degree
    nx = pytest.importorskip("networkx")
    g = _random_graph(250, 1200, seed, directed=True)
    rp, ci = g.csr()
    irp, ici = g.in_csr()
    G = nx.DiGraph()
    G.add_nodes_from(range(250))
    for v in range(250):
        for u in ci[rp[v]:rp[v + 1]]:
            G.add_edge(v, int(u))
    want = nx.core_number(G)
    got = oracle.core_number(rp, ci, directed=True, in_rowptr=irp, in_colidx=ici)
    assert got.tolist() == [want[v] for v in range(250)]


@pytest.mark.parametrize("directed", [False, True])
def test_dependency_mass_identity(directed):
    # sum_v delta_s(v) = sum over reached t != s of (d(s, t) - 1)
    g = _random_graph(120, 240, 7, directed)
    rp, ci, kw = _csr_args(g)
    src = np.arange(120, dtype=np.int32)
    mass, _ = oracle.dependency(rp, ci, src, **kw)
    for s in range(120):
        d = oracle.gdistances(rp, ci, [s]).astype(np.int64)
        reach = d[(d != oracle.UNREACHED32) & (d > 0)]
        assert mass[s] == pytest.approx(float((reach - 1).sum()), rel=1e-12, abs=1e-9)


def test_weighted_accumulation_is_linear():
    g = _random_graph(80, 200, 11)
    rp, ci = g.csr()
    src = np.array([3, 5, 5, 70, 0], np.int32)
    w = np.array([0.5, 2.0, 1.5, 3.0, 0.25])
    _, bw = oracle.dependency(rp, ci, src, w)
    want = sum(wi * oracle.betweenness_raw(rp, ci, [s]) for s, wi in zip(src, w))
    np.testing.assert_allclose(bw, want, rtol=1e-12, atol=1e-12)


def test_oracle_features():
    g = lgbc.SimpleGraph.from_edges(5, [(1, 2), (1, 3), (2, 3), (3, 4)])
    rp, ci = g.csr()
    f = oracle.features(rp, ci)
    deg = np.array([2, 2, 3, 1, 0], float)
    np.testing.assert_allclose(f[:, 0], np.log1p(deg))
    np.testing.assert_allclose(f[:, 1], np.log1p([2, 2, 2, 1, 0]))
    np.testing.assert_allclose(f[2, 2], np.mean(np.log1p([2, 2, 1])))
    np.testing.assert_allclose(f[:, 3], np.log1p([5, 5, 5, 3, 0]))
    assert f[4, 2] == 0.0


def test_mlp_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(size=omlp.NPARAMS) * 0.2
    x = rng.normal(size=(40, 4))
    t = rng.normal(size=40)
    mean, sd = np.array([0.1, -0.2, 0.3, 0.0]), np.array([1.0, 2.0, 0.5, 1.5])
    _, g, _, _ = omlp.loss_and_grad(p, mean, sd, x, t)
    h = 1e-6
    for i in list(rng.choice(omlp.NPARAMS, 60, replace=False)) + [0, omlp.B1, omlp.W2, omlp.B3]:
        q = p.copy()
        q[i] += h
        lp = omlp.loss_and_grad(q, mean, sd, x, t)[0]
        q[i] -= 2 * h
        lm = omlp.loss_and_grad(q, mean, sd, x, t)[0]
        assert (lp - lm) / (2 * h) == pytest.approx(g[i], rel=1e-5, abs=1e-7)


def test_error_metrics():
    exact = np.array([4.0, 3.0, 2.0, 1.0] * 25)
    assert l1_error(exact, exact) == 0.0
    assert l1_error(exact * 1.1, exact) == pytest.approx(0.1)
    assert top_rank_error(exact, exact) == 0.0
    est = exact.copy()
    est[0], est[1] = 0.0, 10.0  # swaps the top-1 vertex
    assert top_rank_error(est, exact) == 1.0


def test_learned_calls_fail_loudly_without_gpu():
    if _lib.lib().lgbc_device_count() > 0:
        pytest.skip("a GPU is present")
    g = lgbc.SimpleGraph.from_edges(3, [(1, 2), (2, 3)])
    with pytest.raises(lgbc.LGBCError):
        lgbc.core_number(g)
    with pytest.raises(lgbc.LGBCError):
        lgbc.SourceProposal()
    with pytest.raises(lgbc.LGBCError):
        lgbc.core_number(lgbc.SimpleDiGraph.from_edges(3, [(1, 2)]))


def test_abi_argument_errors_without_gpu():
    lib = _lib.lib()
    assert lib.lgbc_core_number(None, None) == _lib.LGBC_EINVAL
    assert lib.lgbc_dependency_mass(None, None, 0, None) == _lib.LGBC_EINVAL
    assert lib.lgbc_betweenness_weighted(None, None, None, 0, None) == _lib.LGBC_EINVAL
    assert lib.lgbc_mlp_create(None, 0) == _lib.LGBC_EINVAL
    assert lib.lgbc_mlp_destroy(None) == _lib.LGBC_OK
    assert lib.lgbc_mlp_forward(None, None, 0, None) == _lib.LGBC_EINVAL
    assert lib.lgbc_proposal_sample(None, 0, 0, 0, None, None) == _lib.LGBC_EINVAL
    assert lib.lgbc_tune(None, None) == _lib.LGBC_EINVAL


def _csr_args(g):
    rp, ci = g.csr()
    kw = dict(directed=g.is_directed())
    if g.is_directed():
        irp, ici = g.in_csr()
        kw.update(in_rowptr=irp, in_colidx=ici)
    return rp, ci, kw


def test_core_number_golden_decomposition(known):
    # test/degeneracy.jl:2-6: the reference's decomposition graph and its core numbers
    from conftest import golden_path
    g = lgbc.loadgraph(golden_path("graph-decomposition.lg"))
    rp, ci = g.csr()
    assert oracle.core_number(rp, ci).tolist() == known["core_number"]["expected"]
