"""GPU parity of the learned-proposal path against the oracle: core numbers,
features, exact dependency masses, weighted accumulation, the BF16 / FP32
MLP forward and gradient (checked against the FP64 restatement), training,
the softmax proposal and its sampler, and the gain of the trained proposal
over uniform sampling."""
import numpy as np
import pytest

import lgbc
import lgbc.generators as gen
from lgbc.learned import (SourceProposal, betweenness_centrality_learned,
                          betweenness_raw_weighted, l1_error)
from oracle import mlp as omlp
from oracle import oracle

pytestmark = pytest.mark.gpu


def _random_graph(n, m, seed, directed=False, loops=False):
    rng = np.random.default_rng(seed)
    edges = set()
    while len(edges) < m:
        u, v = (int(a) for a in rng.integers(1, n + 1, size=2))
        if u == v and not loops:
            continue
        edges.add((u, v) if directed else (min(u, v), max(u, v)))
    cls = lgbc.SimpleDiGraph if directed else lgbc.SimpleGraph
    return cls.from_edges(n, sorted(edges))


def _args(g):
    rp, ci = g.csr()
    kw = dict(directed=g.is_directed())
    if g.is_directed():
        irp, ici = g.in_csr()
        kw.update(in_rowptr=irp, in_colidx=ici)
    return rp, ci, kw


GRAPHS = {
    "er": lambda: _random_graph(2000, 8000, 1),
    "sparse": lambda: _random_graph(3000, 2500, 2),  # many components
    "rmat12": lambda: gen.rmat(12, 16, seed=3),
    "ba": lambda: gen.barabasi_albert(3000, 3, seed=4),
    "star": lambda: lgbc.SimpleGraph.from_edges(1200, [(1, v) for v in range(2, 1201)]),
}


@pytest.mark.parametrize("name", sorted(GRAPHS))
def test_core_number_matches_oracle(name):
    g = GRAPHS[name]()
    rp, ci = g.csr()
    np.testing.assert_array_equal(lgbc.core_number(g), oracle.core_number(rp, ci))


def test_core_number_doc_example_and_errors():
    g = lgbc.SimpleGraph.from_edges(6, [(1, 2), (2, 3), (3, 4), (4, 5), (5, 2)])
    assert lgbc.core_number(g).tolist() == [1, 2, 2, 2, 2, 0]
    with pytest.raises(lgbc.ArgumentError):
        lgbc.core_number(lgbc.SimpleGraph.from_edges(3, [(1, 1), (1, 2)]))
    d = _random_graph(800, 4000, 12, directed=True)
    rp, ci = d.csr()
    irp, ici = d.in_csr()
    np.testing.assert_array_equal(
        lgbc.core_number(d), oracle.core_number(rp, ci, directed=True, in_rowptr=irp, in_colidx=ici))
    with pytest.raises(lgbc.MethodError):
        lgbc.features(d)


@pytest.mark.parametrize("name", ["er", "rmat12", "ba", "star"])
def test_features_match_oracle(name):
    g = GRAPHS[name]()
    rp, ci = g.csr()
    np.testing.assert_allclose(lgbc.features(g), oracle.features(rp, ci), rtol=2e-6, atol=2e-6)


def test_features_with_self_loops_use_loop_free_core():
    g = _random_graph(500, 1500, 9, loops=True)
    rp, ci = g.csr()
    assert any(v in ci[rp[v]:rp[v + 1]] for v in range(500))
    f = lgbc.features(g)
    row = np.repeat(np.arange(500), np.diff(rp))
    keep = ci != row
    rp2 = np.concatenate([[0], np.cumsum(np.bincount(row[keep], minlength=500))])
    core = oracle.core_number(rp2, ci[keep])
    np.testing.assert_allclose(f[:, 1], np.log1p(core.astype(np.float64)), rtol=1e-6)


@pytest.mark.parametrize("name,directed", [("er", False), ("sparse", False), ("rmat12", False),
                                           ("ba", False), ("er_dir", True)])
def test_dependency_mass_matches_oracle(name, directed):
    g = _random_graph(1500, 6000, 5, directed=True) if directed else GRAPHS[name]()
    rp, ci, kw = _args(g)
    rng = np.random.default_rng(0)
    src = rng.integers(0, g.nv(), size=150).astype(np.int32)
    src[:3] = src[3]  # repeats
    got = lgbc.dependency_mass(g, src + 1)
    want, _ = oracle.dependency(rp, ci, src, **kw)
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9)
    assert np.all(got == np.round(got))


def test_dependency_mass_isolated_and_all_sources():
    g = lgbc.SimpleGraph.from_edges(70, [(1, 2), (2, 3)])
    m = lgbc.dependency_mass(g)
    assert m[0] == 1.0 and m[2] == 1.0 and m[1] == 0.0 and np.all(m[3:] == 0.0)


@pytest.mark.parametrize("name", ["er", "rmat12", "star"])
def test_weighted_betweenness_matches_oracle(name):
    g = GRAPHS[name]()
    rp, ci = g.csr()
    rng = np.random.default_rng(1)
    src = rng.integers(0, g.nv(), size=200).astype(np.int32)
    src[10:20] = src[0]
    w = rng.uniform(0.1, 5.0, size=200)
    got = betweenness_raw_weighted(g, src, w)
    _, want = oracle.dependency(rp, ci, src, w)
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9 * max(1.0, np.abs(want).max()))


def test_weighted_betweenness_unit_weights_equal_plain():
    g = GRAPHS["rmat12"]()
    src = np.arange(0, g.nv(), 7, dtype=np.int32)
    a = betweenness_raw_weighted(g, src, np.ones(len(src)))
    b = lgbc.betweenness_raw(g, src)
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-9)


def test_weighted_betweenness_wide_path_counts():
    # 50 x 50 grid: path counts pass 2^64, the batch is replayed in FP64
    n = 50
    edges = [(r * n + c + 1, r * n + c + 2) for r in range(n) for c in range(n - 1)]
    edges += [(r * n + c + 1, (r + 1) * n + c + 1) for r in range(n - 1) for c in range(n)]
    g = lgbc.SimpleGraph.from_edges(n * n, edges)
    rp, ci = g.csr()
    src = np.array([0, 2499, 1250, 0], np.int32)
    w = np.array([1.0, 2.0, 0.5, 3.0])
    got = betweenness_raw_weighted(g, src, w)
    _, want = oracle.dependency(rp, ci, src, w)
    np.testing.assert_allclose(got, want, rtol=1e-9)
    assert g.device_handle().stats()["wide_batches"] >= 1


def _bf16_params(m):
    return m.params_bf16().astype(np.float64)


def test_mlp_forward_matches_fp64():
    m = SourceProposal(seed=3)
    m.set_norm([1.0, 0.5, 1.5, 3.0], [0.7, 0.4, 0.6, 1.2])
    rng = np.random.default_rng(0)
    x = rng.normal(size=(5000, 4)).astype(np.float32) + np.array([1.0, 0.5, 1.5, 3.0], np.float32)
    y = m.forward(x)
    mu, sd = m.norm()
    want = omlp.forward(_bf16_params(m), mu.astype(np.float64), sd.astype(np.float64),
                        x.astype(np.float64))
    np.testing.assert_allclose(y, want, rtol=1e-4, atol=1e-4)
    m.close()


@pytest.mark.parametrize("rows", [65, 1000, 4096])
def test_mlp_gradient_matches_fp64(rows):
    m = SourceProposal(seed=11)
    rng = np.random.default_rng(rows)
    p = _bf16_params(m)
    mu, sd = (a.astype(np.float64) for a in m.norm())
    # keep rows away from the ReLU kinks, where FP32 and FP64 agree on every
    # activation pattern
    x = rng.normal(size=(2 * rows, 4)).astype(np.float32)
    _, (_, a1, _, a2, _) = omlp.forward(p, mu, sd, x.astype(np.float64), return_cache=True)
    safe = np.minimum(np.abs(a1).min(1), np.abs(a2).min(1)) > 1e-4
    x = x[safe][:rows]
    assert len(x) == rows
    t = rng.normal(size=rows).astype(np.float32)
    loss, want, _, _ = omlp.loss_and_grad(p, mu, sd, x.astype(np.float64), t.astype(np.float64))
    got, gl = m.grad(x, t)
    assert gl == pytest.approx(loss, rel=1e-4)
    scale = np.abs(want).max()
    np.testing.assert_allclose(got, want, rtol=0, atol=2e-5 * scale)
    m.close()


def test_mlp_training_fits_a_smooth_target():
    rng = np.random.default_rng(5)
    x = rng.normal(size=(16 * 512, 4)).astype(np.float32)
    t = (np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2] + np.abs(x[:, 3])).astype(np.float32)
    off = np.arange(0, len(t) + 1, 512)
    m = SourceProposal(seed=1)
    losses = m.train(x, t, off, steps=1500, batch=512, lr=3e-3, lr_final=3e-4, seed=2)
    assert np.all(np.isfinite(losses))
    assert losses[-100:].mean() < 0.1 * losses[:20].mean()
    # the trained BF16 network, evaluated by the forward kernel
    y = m.forward(x)
    c = (y - t) - (y - t).mean()
    assert float((c * c).mean()) < 0.1 * float(np.var(t))
    m.close()


def test_proposal_matches_softmax_and_sampler():
    g = gen.rmat(11, 8, seed=21)
    m = SourceProposal(seed=4)
    eps = 0.1
    p = m.build(g, eps, return_p=True)
    n = g.nv()
    y = m.forward(lgbc.features(g)).astype(np.float64)
    s = np.exp(y - y.max())
    want = (1 - eps) * s / s.sum() + eps / n
    np.testing.assert_allclose(p, want, rtol=1e-6)
    assert p.sum() == pytest.approx(1.0, abs=1e-12)
    k = 400000
    src, w = m.sample(g, k, seed=9)
    assert src.min() >= 0 and src.max() < n
    np.testing.assert_allclose(w, 1.0 / (k * p[src]), rtol=1e-15)
    counts = np.bincount(src, minlength=n)
    # chi-square of the sampled frequencies against p
    exp_c = k * p
    chi2 = float(((counts - exp_c) ** 2 / exp_c).sum())
    assert chi2 < n + 6 * np.sqrt(2 * n)
    a, _ = m.sample(g, 1000, seed=9)
    b, _ = m.sample(g, 1000, seed=9)
    c, _ = m.sample(g, 1000, seed=10)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    m.close()


def test_systematic_sampling_counts():
    g = gen.rmat(11, 8, seed=22)
    m = SourceProposal(seed=5)
    p = m.build(g, 0.1, return_p=True)
    k = 5000
    src, w = m.sample(g, k, seed=3, scheme="systematic")
    assert np.all(np.diff(src) >= 0)  # draws come in CDF (vertex) order
    counts = np.bincount(src, minlength=g.nv())
    kp = k * p
    assert np.all(counts >= np.floor(kp) - 1) and np.all(counts <= np.ceil(kp) + 1)
    np.testing.assert_allclose(w, 1.0 / (k * p[src]), rtol=1e-15)
    with pytest.raises(lgbc.ArgumentError):
        m.sample(g, 10, scheme="stratified")
    m.close()


def test_weighted_repeats_merge_into_one_lane():
    g = gen.rmat(12, 16, seed=3)
    src = np.array([5, 9, 5, 5, 9, 77], np.int32)
    w = np.array([1.0, 2.0, 0.5, 0.25, 1.0, 3.0])
    a = betweenness_raw_weighted(g, src, w)
    assert g.device_handle().stats()["active_sources"] <= 3
    b = betweenness_raw_weighted(g, np.array([5, 9, 77], np.int32), np.array([1.75, 3.0, 3.0]))
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-9)


def test_importance_estimator_is_unbiased_on_average():
    g = gen.barabasi_albert(600, 2, seed=8)
    exact = lgbc.betweenness_centrality(g)
    m = SourceProposal(seed=2)
    m.build(g, 0.1)
    for scheme in ("iid", "systematic"):
        est = np.mean([betweenness_centrality_learned(g, 64, m, seed=s, build=False, scheme=scheme)
                       for s in range(60)], axis=0)
        assert l1_error(est, exact) < 0.08
    m.close()


def _train_small(seed=0):
    graphs = [gen.rmat(11, 16, seed=100 + i) for i in range(12)]
    graphs += [gen.barabasi_albert(2048, 3, seed=200 + i) for i in range(12)]
    m = SourceProposal(seed=seed)
    info = m.fit(graphs, sources_per_graph=512, steps=800, batch=512, seed=seed)
    return m, info


def test_learned_proposal_beats_uniform_at_equal_samples():
    m, info = _train_small()
    assert info["losses"][-50:].mean() < info["losses"][:10].mean()
    g = gen.rmat(13, 16, seed=999)  # held out
    exact = lgbc.betweenness_centrality(g)
    k = 256
    m.build(g, 0.1)
    l_learned = [l1_error(betweenness_centrality_learned(g, k, m, seed=s, build=False), exact)
                 for s in range(8)]
    rng = np.random.default_rng(7)
    l_uniform = [l1_error(lgbc.betweenness_centrality(g, k, rng=rng), exact) for _ in range(8)]
    assert np.mean(l_learned) < 0.95 * np.mean(l_uniform), (np.mean(l_learned), np.mean(l_uniform))
    m.close()


def test_core_number_golden_decomposition(known):
    from conftest import golden_path
    g = lgbc.loadgraph(golden_path("graph-decomposition.lg"))
    assert lgbc.core_number(g).tolist() == known["core_number"]["expected"]


def _complete(n):
    iu = np.triu_indices(n, 1)
    return lgbc.SimpleGraph.from_edge_arrays(n, iu[0], iu[1])


@pytest.mark.parametrize("name", ["rmat16", "clique1100_with_tail", "hub_digraph"])
def test_core_number_hubs(name):
    # vertices with more than 256 neighbour entries take the block-per-vertex
    # histogram pass; a core number above 1,024 (the 1,100-clique: 1,099)
    # takes its binary-search fallback
    if name == "rmat16":
        g = gen.rmat(16, 16, seed=4)
        kw = {}
    elif name == "clique1100_with_tail":
        k = _complete(1100)
        rp, ci = k.csr()
        src = np.repeat(np.arange(1100), np.diff(rp))
        extra = np.arange(1100, 1400)
        src = np.concatenate([src, extra, extra[1:]])
        dst = np.concatenate([ci, extra % 1100, extra[:-1]])
        g = lgbc.SimpleGraph.from_edge_arrays(1400, src, dst)
        kw = {}
    else:
        rng = np.random.default_rng(9)
        s = np.concatenate([np.zeros(2000, np.int64), rng.integers(1, 3000, 20000)])
        d = np.concatenate([rng.integers(1, 3000, 2000), rng.integers(1, 3000, 20000)])
        keep = s != d
        g = lgbc.SimpleDiGraph.from_edge_arrays(3000, s[keep], d[keep])
        irp, ici = g.in_csr()
        kw = dict(directed=True, in_rowptr=irp, in_colidx=ici)
    rp, ci = g.csr()
    got = lgbc.core_number(g)
    np.testing.assert_array_equal(got, oracle.core_number(rp, ci, **kw))
    if name == "clique1100_with_tail":
        assert got[:1100].min() == 1099
