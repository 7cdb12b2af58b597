"""LightGraphs.Parallel names for the GPU path.

Reference (LightGraphs.jl v1.3.5):
  Parallel.betweenness_centrality(g, vs|k, distmx; normalize, endpoints,
      parallel=:distributed|:threads)   src/Parallel/centrality/betweenness.jl:1-7
  Parallel.gdistances(g, source(s); queue_segment_size=20)
      src/Parallel/traversals/gdistances.jl:118-139
  Parallel.gdistances!(g, source(s), vert_level; queue_segment_size=20)  :36-116
The results equal the serial functions' (the reference's own tests assert
that, test/parallel/centrality/betweenness.jl, test/parallel/traversals/
gdistances.jl); on one GPU the ``parallel`` and ``queue_segment_size``
keywords select nothing and are accepted for compatibility.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from . import centrality as _c
from . import traversals as _t

_PARALLEL_MODES = ("distributed", "threads", ":distributed", ":threads")


def betweenness_centrality(g, vs=None, distmx=None, *, normalize: bool = True,
                           endpoints: bool = False, parallel: str = "distributed",
                           rng=None) -> np.ndarray:
    """Drop-in for Parallel.betweenness_centrality (either ``parallel`` mode)."""
    if str(parallel) not in _PARALLEL_MODES:
        raise _lib.ArgumentError(f"unknown parallel mode {parallel!r}")
    return _c.betweenness_centrality(g, vs, distmx, normalize=normalize, endpoints=endpoints,
                                     rng=rng)


def gdistances(g, sources, *, queue_segment_size: int = 20) -> np.ndarray:
    """Drop-in for Parallel.gdistances."""
    return _t.gdistances(g, sources)


def gdistances_(g, sources, vert_level: np.ndarray, *, queue_segment_size: int = 20) -> np.ndarray:
    """Parallel.gdistances! fills vert_level with typemax first
    (src/Parallel/traversals/gdistances.jl:47), then writes the levels."""
    vert_level[:] = _t._typemax(vert_level.dtype)
    return _t.gdistances_(g, sources, vert_level)
