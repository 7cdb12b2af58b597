"""GPU parity of the degree-binned top-down BFS (gdistances).

A top-down level walks the out-lists of 32 frontier vertices per warp as one
concatenation and defers vertices with more than 1,024 out-edges to a kernel
in which the whole grid walks each such list.  These graphs put vertices on
both sides of that cut into the frontier, with every level forced top-down
(and once with the default direction choice), against the oracle's
gdistances! (src/traversals/bfs.jl:95-124) bit for bit.
"""
import numpy as np
import pytest

import lgbc
from lgbc import generators as G
from conftest import csr_args
from oracle import oracle

pytestmark = pytest.mark.gpu


def star_with_tails():
    # a 5,000-leaf star, a 1,025-leaf star (just past the cut) joined to it,
    # a 1,024-leaf one (just below) and a path hanging off a leaf
    edges = [(0, i) for i in range(1, 5001)]
    edges += [(5001, i) for i in range(5002, 6027)] + [(4999, 5001)]
    edges += [(6027, i) for i in range(6028, 7052)] + [(6026, 6027)]
    edges += [(7052 + i, 7053 + i) for i in range(200)] + [(3, 7052)]
    e = np.asarray(edges)
    return lgbc.SimpleGraph.from_edge_arrays(7253, e[:, 0], e[:, 1])


def directed_hub():
    rng = np.random.default_rng(2)
    src = np.concatenate([np.zeros(3000, np.int64), rng.integers(1, 4000, 6000)])
    dst = np.concatenate([rng.integers(1, 4000, 3000), rng.integers(1, 4000, 6000)])
    keep = src != dst
    return lgbc.SimpleDiGraph.from_edge_arrays(4000, src[keep], dst[keep])


GRAPHS = {
    "star_with_tails": star_with_tails,
    "rmat18": lambda: G.rmat(18, 16, seed=7),
    "rmat16_directed": lambda: G.rmat(16, 16, seed=8, directed=True),
    "directed_hub": directed_hub,
}


@pytest.mark.parametrize("name", sorted(GRAPHS))
@pytest.mark.parametrize("direction", ["topdown", "auto"])
def test_binned_topdown_matches_oracle(name, direction):
    g = GRAPHS[name]()
    rp, ci, _ = csr_args(g)
    deg = np.diff(rp)
    assert deg.max() > 1024  # the grid-wide kernel runs
    h = g.device_handle()
    if direction == "topdown":
        h.set_tuning(alpha=1e-12, beta=1e12)
    try:
        rng = np.random.default_rng(3)
        hubs = np.flatnonzero(deg > 1024)
        for srcs in ([0], [int(hubs[0])], [1, 2, 3], rng.choice(g.nv(), 25).tolist()):
            got = lgbc.gdistances(g, [s + 1 for s in srcs]).astype(np.int64)
            exp = oracle.gdistances(rp, ci, srcs).astype(np.int64)
            exp[exp == oracle.UNREACHED32] = np.iinfo(g.eltype).max
            assert np.array_equal(got, exp), srcs
    finally:
        h.set_tuning(alpha=14.0, beta=24.0)
