"""gdistances / gdistances! with LightGraphs' semantics, computed by the CUDA library.

Reference: src/traversals/bfs.jl (LightGraphs.jl v1.3.5)
  gdistances!(g, source, vert_level; sort_alg=QuickSort)   :95-124
  gdistances(g, source; sort_alg=QuickSort)                :141
  bfs_parents / bfs_tree / tree                            :10-19, :35-76
  has_path(g, u, v; exclude_vertices)                      :150-172
and, from src/shortestpaths/dijkstra.jl:59-141 (unit weights),
  dijkstra_shortest_paths(g, s).pathcounts / .dists        path_counts
``source`` is one vertex or a collection (a multi-source BFS: distance to the
nearest source).  Unreachable vertices hold typemax(eltype(g)).  The
``sort_alg`` keyword only orders the reference's level queue and is accepted
and ignored.
"""
from __future__ import annotations

import ctypes
import numbers

import numpy as np

from . import _lib
from .centrality import _sources0


def _typemax(dtype) -> int:
    return int(np.iinfo(dtype).max)


def _as_sources(g, source) -> np.ndarray:
    if isinstance(source, numbers.Integral) and not isinstance(source, bool):
        return _sources0(g, [int(source)])
    return _sources0(g, source)


def _device_levels(g, src0: np.ndarray) -> np.ndarray:
    """int32 levels from the GPU BFS; INT32_MAX marks unreached."""
    out = np.empty(g.nv(), np.int32)
    if g.nv() == 0:
        return out
    h = g.device_handle()
    src = np.ascontiguousarray(src0, np.int32)
    _lib.check(_lib.lib().lgbc_gdistances(h.handle, _lib.ptr(src), len(src), _lib.ptr(out)))
    return out


def _to_eltype(levels: np.ndarray, dtype) -> np.ndarray:
    out = levels.astype(dtype)
    out[levels == _lib.UNREACHED] = _typemax(dtype)
    return out


def gdistances(g, source, *, sort_alg=None) -> np.ndarray:
    """Drop-in for LightGraphs.gdistances (bfs.jl:141)."""
    lv = _device_levels(g, _as_sources(g, source))
    return _to_eltype(lv, g.eltype)


def gdistances_(g, source, vert_level: np.ndarray, *, sort_alg=None) -> np.ndarray:
    """gdistances!(g, source, vert_level) (bfs.jl:95-124): writes the level of
    every vertex the BFS reaches and leaves the other entries as they are
    (callers pre-fill them with typemax, as gdistances does)."""
    if len(vert_level) != g.nv():
        raise _lib.ArgumentError("vert_level must have nv(g) entries")
    lv = _device_levels(g, _as_sources(g, source))
    reached = lv != _lib.UNREACHED
    vert_level[reached] = lv[reached].astype(vert_level.dtype)
    return vert_level


def multi_gdistances(g, sources) -> np.ndarray:
    """One independent single-source gdistances per entry of ``sources``,
    as a (len(sources), nv(g)) matrix in eltype(g).  The GPU runs up to 64 of
    them as bit lanes of one BFS (lgbc_gdistances_batch)."""
    src = _sources0(g, sources)
    n = g.nv()
    out = np.empty((len(src), n), np.int32)
    if len(src) and n:
        h = g.device_handle()
        _lib.check(_lib.lib().lgbc_gdistances_batch(h.handle, _lib.ptr(src), len(src),
                                                    _lib.ptr(out)))
    return _to_eltype(out, g.eltype)


def bfs_parents(g, s: int, *, dir: str = "out") -> np.ndarray:
    """Drop-in for bfs_parents(g, s; dir=:out) (src/traversals/bfs.jl:35-66):
    1-based parent of every vertex (the smallest neighbour one level closer,
    as the reference's sorted levels choose), s for s, 0 where unreached."""
    d = {"out": 0, ":out": 0, "in": 1, ":in": 1}.get(str(dir))
    if d is None:
        raise _lib.ArgumentError(f"dir must be :out or :in, got {dir!r}")
    src = _sources0(g, [s])
    out = np.empty(g.nv(), np.int32)
    _lib.check(_lib.lib().lgbc_bfs_parents(g.device_handle().handle, int(src[0]), d,
                                           _lib.ptr(out)))
    return (out.astype(np.int64) + 1).astype(g.eltype)


def tree(parents):
    """tree(parents) (src/traversals/bfs.jl:10-19): the DiGraph with an
    edge u -> v for every v whose parent u is neither 0 nor v itself."""
    from .graphs import SimpleDiGraph
    p = np.asarray(parents, np.int64)
    v = np.arange(1, len(p) + 1)
    keep = (p > 0) & (p != v)
    return SimpleDiGraph.from_edge_arrays(len(p), p[keep] - 1, v[keep] - 1, eltype=p.dtype)


def bfs_tree(g, s: int, *, dir: str = "out"):
    """Drop-in for bfs_tree(g, s; dir) = tree(bfs_parents(g, s; dir)) (bfs.jl:76)."""
    return tree(bfs_parents(g, s, dir=dir))


def has_path(g, u: int, v: int, *, exclude_vertices=()) -> bool:
    """Drop-in for has_path(g, u, v; exclude_vertices) (bfs.jl:150-172)."""
    uv = _sources0(g, [u, v])
    ex = np.ascontiguousarray(_sources0(g, list(exclude_vertices)), np.int32)
    res = ctypes.c_int()
    _lib.check(_lib.lib().lgbc_has_path(g.device_handle().handle, int(uv[0]), int(uv[1]),
                                        _lib.ptr(ex) if len(ex) else None, len(ex),
                                        ctypes.byref(res)))
    return bool(res.value)


def path_counts(g, sources):
    """DijkstraState.pathcounts and .dists of dijkstra_shortest_paths(g, s)
    with unit weights (src/shortestpaths/dijkstra.jl:59-141), one row per
    entry of ``sources`` (1-based): (pathcounts float64 (len, nv),
    dists eltype(g) (len, nv)).  pathcounts is 1 at the source and 0 where
    the source does not reach; counts below 2^53 are exact, larger ones are
    the exact count rounded to the nearest Float64.  dists holds
    typemax(eltype(g)) where the source does not reach."""
    src = _sources0(g, sources)
    n = g.nv()
    pc = np.zeros((len(src), n), np.float64)
    dist = np.empty((len(src), n), np.int32)
    if len(src) and n:
        h = g.device_handle()
        _lib.check(_lib.lib().lgbc_path_counts(h.handle, _lib.ptr(src), len(src), _lib.ptr(pc),
                                               _lib.ptr(dist)))
    else:
        dist.fill(_lib.UNREACHED)
    return pc, _to_eltype(dist, g.eltype)
