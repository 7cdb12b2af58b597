"""LightGraphs.Parallel names for the GPU path.

Reference (LightGraphs.jl v1.3.5):
  Parallel.betweenness_centrality(g, vs|k, distmx; normalize, endpoints,
      parallel=:distributed|:threads)   src/Parallel/centrality/betweenness.jl:1-7
  Parallel.gdistances(g, source(s); queue_segment_size=20)
      src/Parallel/traversals/gdistances.jl:118-139
  Parallel.gdistances!(g, source(s), vert_level; queue_segment_size=20)  :36-116
  Parallel.stress_centrality(g, vs|k; parallel)  src/Parallel/centrality/stress.jl:1-6
  Parallel.bfs_tree(g, s)                     src/Parallel/traversals/bfs.jl:94-104
  Parallel.closeness_centrality(g, distmx; normalize, parallel)
      src/Parallel/centrality/closeness.jl:1-3
  Parallel.radiality_centrality(g; parallel)  src/Parallel/centrality/radiality.jl:1-2
  Parallel.eccentricity / diameter / radius / periphery / center
      src/Parallel/distance.jl:3-34
The results equal the serial functions' (the reference's own tests assert
that, test/parallel/centrality/betweenness.jl, test/parallel/traversals/
gdistances.jl); on one GPU the ``parallel`` and ``queue_segment_size``
keywords select nothing and are accepted for compatibility.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from . import centrality as _c
from . import distance as _d
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


def closeness_centrality(g, distmx=None, *, normalize: bool = True,
                         parallel: str = "distributed") -> np.ndarray:
    """Drop-in for Parallel.closeness_centrality (either ``parallel`` mode)."""
    if str(parallel) not in _PARALLEL_MODES:
        raise _lib.ArgumentError(f"unknown parallel mode {parallel!r}")
    return _d.closeness_centrality(g, distmx, normalize=normalize)


def radiality_centrality(g, *, parallel: str = "distributed") -> np.ndarray:
    """Drop-in for Parallel.radiality_centrality (either ``parallel`` mode)."""
    if str(parallel) not in _PARALLEL_MODES:
        raise _lib.ArgumentError(f"unknown parallel mode {parallel!r}")
    return _d.radiality_centrality(g)


def eccentricity(g, vs=None, distmx=None) -> np.ndarray:
    """Drop-in for Parallel.eccentricity (a vector, warning once if infinite)."""
    import warnings
    with warnings.catch_warnings(record=True) as caught:
        warnings.simplefilter("always")
        e = _d.eccentricity(g, vs, distmx)
    if caught:
        warnings.warn("Infinite path length detected")
    return np.atleast_1d(e)


def diameter(g, distmx=None):
    return int(np.max(eccentricity(g, None, distmx)))


def radius(g, distmx=None):
    return int(np.min(eccentricity(g, None, distmx)))


def periphery(g, distmx=None) -> list:
    return _d.periphery(eccentricity(g, None, distmx))


def center(g, distmx=None) -> list:
    return _d.center(eccentricity(g, None, distmx))


def stress_centrality(g, vs=None, *, parallel: str = "distributed", rng=None) -> np.ndarray:
    """Drop-in for Parallel.stress_centrality (either ``parallel`` mode)."""
    if str(parallel) not in _PARALLEL_MODES:
        raise _lib.ArgumentError(f"unknown parallel mode {parallel!r}")
    return _c.stress_centrality(g, vs, rng=rng)


def bfs_tree(g, s: int, nv: int | None = None):
    """Drop-in for Parallel.bfs_tree(g, s[, nv]).  The threaded reference lets
    any discoverer win; the GPU returns the serial bfs_tree's parents, which
    is one of the trees the reference may return."""
    return _t.bfs_tree(g, s)
