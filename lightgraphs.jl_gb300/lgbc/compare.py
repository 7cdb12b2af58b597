"""Uniform versus learned source sampling, judged against exact betweenness.

The harness behind the learned-proposal workload: it trains the default
proposal on generated graphs, cuts held-out evaluation graphs, runs both
estimators at several sample budgets and seeds, and reports L1 and top-1 %
rank error together with GPU time (CUDA events on the graph's stream).

* uniform -- ``betweenness_centrality(g, k)``: k distinct sources from
  ``sample`` (src/utils.jl:12-45), rescaled by n/k (betweenness.jl:77-78).
* learned -- ``betweenness_centrality_learned``: k i.i.d. sources from the
  proposal, weights 1/(k p), rescaled with k = n.

* ceiling arms -- i.i.d. draws from proposals built from exact per-source
  information that a predictor can at best reproduce: p proportional to the
  exact dependency mass (a perfect prediction of the network's target), to
  its square root, and uniform over the non-isolated sources.

"Equal error" compares, for every uniform budget k_u, the learned budget k_l
at which the learned estimator's mean L1 error equals uniform's at k_u
(log-log interpolation between measured budgets); both estimators' GPU time is
linear in k, so the time at k_l is interpolated the same way.
"""
from __future__ import annotations

import ctypes
import math
import time

import numpy as np

from . import _lib
from . import generators as gen
from .centrality import _rescale_, betweenness_centrality, sample
from .graphs import SimpleGraph
from .learned import (SourceProposal, betweenness_centrality_learned, betweenness_raw_weighted,
                      dependency_mass, l1_error, top_rank_error)
from .traversals import gdistances


class _Timer:
    """CUDA-event time of everything a graph handle queued between start and stop."""

    def __init__(self, g):
        self.h = g.device_handle().handle

    def __enter__(self):
        _lib.check(_lib.lib().lgbc_timer_start(self.h))
        return self

    def __exit__(self, *exc):
        ms = ctypes.c_double()
        launches = ctypes.c_int64()
        _lib.check(_lib.lib().lgbc_timer_stop(self.h, ctypes.byref(ms), ctypes.byref(launches)))
        self.ms = float(ms.value)
        self.launches = int(launches.value)
        return False


def training_graphs(n_rmat: int = 128, n_ba: int = 128, scale: int = 14, seed0: int = 10000):
    """R-MAT (edge factor 16, a/b/c = .57/.19/.19) and Barabasi-Albert (k = 3)
    graphs of 2^scale vertices, seeds seed0, seed0 + 1, ..."""
    gs = [gen.rmat(scale, 16, seed=seed0 + i) for i in range(n_rmat)]
    gs += [gen.barabasi_albert(2 ** scale, 3, seed=seed0 + n_rmat + i) for i in range(n_ba)]
    return gs


def train_default(graphs=None, *, sources_per_graph: int = 1024, steps: int = 3000,
                  batch: int = 1024, seed: int = 0):
    """The default proposal: trained on ``training_graphs()``; returns
    (proposal, info) with the generation / target / training wall times."""
    t0 = time.perf_counter()
    if graphs is None:
        graphs = training_graphs()
    t1 = time.perf_counter()
    m = SourceProposal(seed=seed)
    info = m.fit(graphs, sources_per_graph=sources_per_graph, steps=steps, batch=batch, seed=seed)
    t2 = time.perf_counter()
    losses = info.pop("losses")
    info.update(generate_s=t1 - t0, fit_s=t2 - t1, loss_first=float(losses[:20].mean()),
                loss_last=float(losses[-100:].mean()), steps=steps, batch=batch,
                sources_per_graph=sources_per_graph)
    return m, info


def bfs_ball(g, center0: int, size: int):
    """Induced subgraph on the `size` vertices closest to `center0` (0-based;
    ties by vertex id), vertices kept in id order.  Returns (subgraph,
    0-based original ids)."""
    d0 = gdistances(g, center0 + 1)
    reach = np.flatnonzero(d0 != np.iinfo(d0.dtype).max)
    d = d0.astype(np.int64)
    order = reach[np.lexsort((reach, d[reach]))]
    keep = np.sort(order[:size])
    n = g.nv()
    newid = np.full(n, -1, np.int64)
    newid[keep] = np.arange(len(keep))
    rp, ci = g.csr()
    starts, ends = rp[keep], rp[keep + 1]
    lens = ends - starts
    idx = np.repeat(starts - np.concatenate([[0], np.cumsum(lens)[:-1]]), lens) + np.arange(lens.sum())
    nbr = newid[ci[idx]]
    row = np.repeat(np.arange(len(keep)), lens)
    ok = nbr >= 0
    counts = np.bincount(row[ok], minlength=len(keep))
    sub_rp = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    sub = SimpleGraph.from_csr(sub_rp, nbr[ok].astype(np.int32), eltype=np.int32)
    return sub, keep.astype(np.int64)


def exact(g):
    """Exact normalised betweenness and its GPU milliseconds."""
    with _Timer(g) as t:
        b = betweenness_centrality(g)
    return b, t.ms


def run_estimators(g, exact_bc, proposal: SourceProposal, ks_uniform, ks_learned, seeds=8,
                   eps: float = 0.1, seed0: int = 100):
    """Per-run records (method, k, seed, l1, top1, gpu_ms) plus the learned
    proposal's build time (features, MLP, softmax, CDF)."""
    recs = []
    for k in ks_uniform:
        for s in range(seeds):
            src = np.asarray(sample(g.vertices(), int(k), rng=np.random.default_rng(seed0 + s)))
            with _Timer(g) as t:
                b = betweenness_centrality(g, src)
            # betweenness_centrality(g, vs) rescales by n / len(vs) like the k form
            recs.append(dict(method="uniform", k=int(k), seed=s, l1=l1_error(b, exact_bc),
                             top1=top_rank_error(b, exact_bc), gpu_ms=t.ms))
    with _Timer(g) as t:
        proposal.build(g, eps)
    build_ms = t.ms
    for method, scheme in (("learned", "iid"), ("learned_systematic", "systematic")):
        for k in ks_learned:
            for s in range(seeds):
                with _Timer(g) as t:
                    b = betweenness_centrality_learned(g, int(k), proposal, eps=eps,
                                                       seed=seed0 + s, build=False, scheme=scheme)
                recs.append(dict(method=method, k=int(k), seed=s, l1=l1_error(b, exact_bc),
                                 top1=top_rank_error(b, exact_bc), gpu_ms=t.ms))
    return recs, build_ms


def ceiling_proposals(g):
    """Proposals from exact per-source information: ``mass`` (p proportional
    to sum_v delta_s(v)), ``sqrt_mass`` and ``uniform_active`` (uniform over
    vertices with an edge), plus the GPU milliseconds of the exact masses."""
    with _Timer(g) as t:
        mass = dependency_mass(g)
    out = {}
    for name, w in (("mass", mass), ("sqrt_mass", np.sqrt(mass)),
                    ("uniform_active", (g.degrees() > 0).astype(np.float64))):
        if w.sum() > 0:  # a graph without paths of length 2 has no mass to sample by
            out[name] = w / w.sum()
    return out, t.ms


def run_fixed(g, exact_bc, p, ks, method: str, seeds=8, seed0=100):
    """Records for k i.i.d. draws from the fixed proposal p (drawn on the
    host) with weights 1/(k p), through the weighted Brandes call; GPU time
    covers that call only."""
    n = g.nv()
    recs = []
    for k in ks:
        for s in range(seeds):
            rng = np.random.default_rng(seed0 + s)
            src = rng.choice(n, size=int(k), p=p).astype(np.int32)
            w = 1.0 / (int(k) * p[src])
            with _Timer(g) as t:
                b = betweenness_raw_weighted(g, src, w)
            _rescale_(b, n, True, g.is_directed(), n)
            recs.append(dict(method=method, k=int(k), seed=s, l1=l1_error(b, exact_bc),
                             top1=top_rank_error(b, exact_bc), gpu_ms=t.ms))
    return recs


def _means(recs, method):
    ks = sorted({r["k"] for r in recs if r["method"] == method})
    out = []
    for k in ks:
        rs = [r for r in recs if r["method"] == method and r["k"] == k]
        out.append(dict(k=k, l1=float(np.mean([r["l1"] for r in rs])),
                        l1_sd=float(np.std([r["l1"] for r in rs])),
                        top1=float(np.mean([r["top1"] for r in rs])),
                        gpu_ms=float(np.median([r["gpu_ms"] for r in rs]))))
    return out


def _interp_loglog(xs, ys, y):
    """x where the piecewise log-log line through (xs, ys) (ys decreasing)
    reaches y; extrapolates from the end segments."""
    lx, ly = np.log(np.asarray(xs, float)), np.log(np.asarray(ys, float))
    t = math.log(y)
    for i in range(len(lx) - 1):
        if (ly[i] - t) * (ly[i + 1] - t) <= 0 and ly[i] != ly[i + 1]:
            f = (t - ly[i]) / (ly[i + 1] - ly[i])
            return float(math.exp(lx[i] + f * (lx[i + 1] - lx[i])))
    i = 0 if t > ly[0] else len(lx) - 2
    slope = (ly[i + 1] - ly[i]) / (lx[i + 1] - lx[i]) if lx[i + 1] != lx[i] else -0.5
    if slope == 0:
        return float("nan")
    return float(math.exp(lx[i] + (t - ly[i]) / slope))


def _interp_lin(xs, ys, x):
    return float(np.interp(x, xs, ys, left=None, right=None)) if xs[0] <= x <= xs[-1] else \
        float(ys[0] + (ys[-1] - ys[0]) * (x - xs[0]) / (xs[-1] - xs[0]))


def summarise(recs, build_ms: float, k_targets,
              methods=("learned", "learned_systematic")):
    """Mean errors per budget and, per method, the equal-error GPU-time
    comparison against uniform sampling (``equal_error`` for "learned",
    ``equal_error_<method>`` for the others; ``build_ms`` is added to the
    learned methods only)."""
    uni = _means(recs, "uniform")
    out = dict(uniform=uni, build_ms=build_ms)
    for method in methods:
        lrn = _means(recs, method)
        if not lrn:
            continue
        lk = [r["k"] for r in lrn]
        table = []
        for ku in k_targets:
            u = next(r for r in uni if r["k"] == ku)
            kl = _interp_loglog(lk, [r["l1"] for r in lrn], u["l1"])
            tl = _interp_lin(lk, [r["gpu_ms"] for r in lrn], kl)
            bm = build_ms if method.startswith("learned") else 0.0
            table.append(dict(k_uniform=ku, l1_uniform=u["l1"], top1_uniform=u["top1"],
                              ms_uniform=u["gpu_ms"], k_learned_equal_l1=kl, ms_learned=tl,
                              ms_learned_with_build=tl + bm,
                              time_ratio=tl / u["gpu_ms"],
                              time_ratio_with_build=(tl + bm) / u["gpu_ms"]))
        out[method] = lrn
        key = {"learned": "equal_error", "learned_systematic": "equal_error_systematic"}
        out[key.get(method, "equal_error_" + method)] = table
    return out
