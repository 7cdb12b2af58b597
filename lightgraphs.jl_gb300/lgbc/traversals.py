"""gdistances / gdistances! with LightGraphs' semantics, computed by the CUDA library.

Reference: src/traversals/bfs.jl (LightGraphs.jl v1.3.5)
  gdistances!(g, source, vert_level; sort_alg=QuickSort)   :95-124
  gdistances(g, source; sort_alg=QuickSort)                :141
``source`` is one vertex or a collection (a multi-source BFS: distance to the
nearest source).  Unreachable vertices hold typemax(eltype(g)).  The
``sort_alg`` keyword only orders the reference's level queue and is accepted
and ignored.
"""
from __future__ import annotations

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
