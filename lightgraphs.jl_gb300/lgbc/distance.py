"""Distance-based centralities and measures on the GPU's multi-source BFS.

Reference (LightGraphs.jl v1.3.5), all with unit weights (``weights(g)``):
  closeness_centrality(g, distmx; normalize=true)  src/centrality/closeness.jl:33-55
  radiality_centrality(g)                          src/centrality/radiality.jl:36-49
  eccentricity(g[, v | vs][, distmx])              src/distance.jl:73-84
  diameter / radius / periphery / center           src/distance.jl:86-170
Each runs one unit-weight Dijkstra per vertex and reduces its distance
vector.  Here the vertices run as bit lanes of the multi-source BFS
(lgbc_distance_stats), which returns, per source, the reachable count, the
distance sum and the largest distance; the host finishes each metric with the
reference's own arithmetic, including its Int64 handling of typemax(Int)
distances for unreachable vertices.
"""
from __future__ import annotations

import warnings

import numpy as np

from . import _lib
from .centrality import _check_distmx, _sources0

TYPEMAX = np.iinfo(np.int64).max


def distance_stats(g, src0: np.ndarray):
    """(reached incl. the source, distance sum, largest distance) per 0-based source."""
    src = np.ascontiguousarray(src0, np.int32)
    k = len(src)
    reached = np.zeros(k, np.int64)
    dsum = np.zeros(k, np.int64)
    dmax = np.zeros(k, np.int32)
    if k:
        _lib.check(_lib.lib().lgbc_distance_stats(g.device_handle().handle, _lib.ptr(src), k,
                                                  _lib.ptr(reached), _lib.ptr(dsum),
                                                  _lib.ptr(dmax)))
    return reached, dsum, dmax


def closeness_centrality(g, distmx=None, *, normalize: bool = True) -> np.ndarray:
    """closeness_centrality (closeness.jl:33-55): for u with degree > 0,
    l / sum(d) over the reachable set (l = reachable - 1), times l / (n - 1)
    when normalising; 0.0 otherwise."""
    _check_distmx(g, distmx)
    n = g.nv()
    out = np.zeros(n, np.float64)
    act = np.flatnonzero(g.degrees() > 0).astype(np.int32)
    reached, dsum, _ = distance_stats(g, act)
    for u, r, s in zip(act.tolist(), reached.tolist(), dsum.tolist()):
        l = r - 1
        if s > 0:
            c = l / s
            if normalize:
                c *= l / (n - 1)
            out[u] = c
    return out


def _ecc_int(n: int, reached: np.ndarray, dmax: np.ndarray) -> np.ndarray:
    """maximum(dists) as Int64: typemax(Int) when some vertex is unreachable."""
    return np.where(reached < n, TYPEMAX, dmax.astype(np.int64))


def radiality_centrality(g) -> np.ndarray:
    """radiality_centrality (radiality.jl:36-49).  sum(d.dists) is an Int64
    sum that counts typemax(Int) for every unreachable vertex and wraps, as
    the reference's does; dmtr is the largest distance (typemax(Int) when the
    graph is not strongly connected) as a Float64."""
    n = g.nv()
    if n == 0:
        return np.zeros(0, np.float64)
    reached, dsum, dmax = distance_stats(g, np.arange(n, dtype=np.int32))
    wrapped = (dsum.astype(np.uint64) + (n - reached).astype(np.uint64) * np.uint64(TYPEMAX))
    total = wrapped.view(np.int64)
    meandists = total.astype(np.float64) / float(n - 1) if n > 1 else \
        np.full(n, np.nan)  # sum(d) / 0 = NaN for the lone vertex (0 / 0)
    dmtr = max(0.0, float(_ecc_int(n, reached, dmax).max()))
    return ((dmtr + 1) - meandists) / dmtr if dmtr != 0 else ((dmtr + 1) - meandists) / 0.0


def eccentricity(g, vs=None, distmx=None):
    """eccentricity(g, v) -> Int; eccentricity(g, vs=vertices(g)) -> Vector.
    Unreachable vertices give typemax(Int) with the reference's warning."""
    _check_distmx(g, distmx)
    n = g.nv()
    scalar = isinstance(vs, (int, np.integer)) and not isinstance(vs, bool)
    src = np.arange(n, dtype=np.int32) if vs is None else _sources0(g, [vs] if scalar else vs)
    reached, _, dmax = distance_stats(g, src)
    e = _ecc_int(n, reached, dmax)
    for v in src[e == TYPEMAX].tolist():
        warnings.warn(f"Infinite path length detected for vertex {v + 1}")
    return int(e[0]) if scalar else e


def diameter(g_or_eccs, distmx=None):
    """diameter(eccentricities) or diameter(g): the largest eccentricity."""
    e = g_or_eccs if isinstance(g_or_eccs, np.ndarray) else eccentricity(g_or_eccs, None, distmx)
    return int(np.max(e))


def radius(g_or_eccs, distmx=None):
    """radius(eccentricities) or radius(g): the smallest eccentricity."""
    e = g_or_eccs if isinstance(g_or_eccs, np.ndarray) else eccentricity(g_or_eccs, None, distmx)
    return int(np.min(e))


def periphery(g_or_eccs, distmx=None) -> list:
    """1-based vertices whose eccentricity equals the diameter."""
    e = g_or_eccs if isinstance(g_or_eccs, np.ndarray) else eccentricity(g_or_eccs, None, distmx)
    return (np.flatnonzero(e == np.max(e)) + 1).tolist()


def center(g_or_eccs, distmx=None) -> list:
    """1-based vertices whose eccentricity equals the radius."""
    e = g_or_eccs if isinstance(g_or_eccs, np.ndarray) else eccentricity(g_or_eccs, None, distmx)
    return (np.flatnonzero(e == np.min(e)) + 1).tolist()
