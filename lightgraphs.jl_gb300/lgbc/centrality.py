"""betweenness_centrality with LightGraphs' signature, computed by the CUDA library.

Reference: src/centrality/betweenness.jl and src/centrality/stress.jl
(LightGraphs.jl v1.3.5).
  betweenness_centrality(g, vs=vertices(g), distmx=weights(g); normalize=true,
                         endpoints=false)                          :46-75
  betweenness_centrality(g, k::Integer, distmx=weights(g); ...)    :77-78
  _rescale!(betweenness, n, normalize, directed, k)                :136-160
The source loop, Dijkstra state and accumulation (:57-68, :81-134) run on the
GPU (lgbc_betweenness); sampling and the rescale stay on the host exactly as
the reference does them.
"""
from __future__ import annotations

import ctypes
import numbers

import numpy as np

from . import _lib
from .graphs import DefaultDistance


def _check_distmx(g, distmx) -> None:
    if distmx is None:
        return
    if isinstance(distmx, DefaultDistance) and distmx.nv == g.nv():
        return
    raise _lib.MethodError(
        "betweenness_centrality on the GPU covers unit weights only "
        "(distmx must be weights(g) = DefaultDistance)")


def _is_count(x) -> bool:
    return isinstance(x, numbers.Integral) and not isinstance(x, bool)


def _rng(rng):
    if rng is None:
        return np.random.default_rng()
    if isinstance(rng, np.random.Generator):
        return rng
    return np.random.default_rng(rng)


def sample_(a: list, k: int, rng=None, exclude=()) -> list:
    """sample!(rng, a, k; exclude) -- src/utils.jl:12-28: k distinct elements
    by a partial Fisher-Yates shuffle that swaps each pick to the end of `a`
    (mutates `a`).  Raises ArgumentError when len(a) < k + len(exclude)."""
    minsize = k + len(exclude)
    if len(a) < minsize:
        raise _lib.ArgumentError(f"vector must be at least size {minsize}")
    r_ = _rng(rng)
    res = []
    n = len(a)
    i = 1
    excl = set(exclude)
    while len(res) < k:
        r = int(r_.integers(1, n - i + 2))  # rand(rng, 1:(n - i + 1))
        if a[r - 1] not in excl:
            res.append(a[r - 1])
            a[r - 1], a[n - i] = a[n - i], a[r - 1]
            i += 1
    return res


def sample(a, k: int, rng=None, exclude=()) -> list:
    """sample(a, k) -- src/utils.jl:43: sample! on a copy."""
    return sample_(list(a), k, rng=rng, exclude=exclude)


def _rescale_(betweenness: np.ndarray, n: int, normalize: bool, directed: bool, k: int) -> None:
    """_rescale! (src/centrality/betweenness.jl:136-160), in place.
    (n - 1) * (n - 2) is an Int64 product in Julia (nv(g)::T promotes with the
    Int64 literals), so it cannot overflow here either."""
    do_scale = False
    scale = 1.0
    if normalize:
        if n <= 2:
            do_scale = False
        else:
            do_scale = True
            scale = 1.0 / float((n - 1) * (n - 2))
    else:
        if not directed:
            do_scale = True
            scale = 1.0 / 2.0
        else:
            do_scale = False
    if do_scale:
        if k > 0:
            scale = scale * float(n) / float(k)
        betweenness *= scale


def _sources0(g, vs) -> np.ndarray:
    """1-based vertex collection -> int32 0-based array, with BoundsError."""
    if isinstance(vs, range) and vs.step == 1 and len(vs) > 0:
        lo, hi = vs.start, vs.stop - 1
        if lo < 1 or hi > g.nv():
            raise _lib.BoundsError(f"vertices {lo}:{hi} outside 1:{g.nv()}")
        return np.arange(lo - 1, hi, dtype=np.int32)
    a = np.asarray(list(vs) if not isinstance(vs, np.ndarray) else vs).ravel()
    if a.size == 0:
        return np.zeros(0, np.int32)
    if not np.issubdtype(a.dtype, np.integer):
        raise _lib.ArgumentError("vertex ids must be integers")
    a = a.astype(np.int64)
    if a.min() < 1 or a.max() > g.nv():
        bad = a[(a < 1) | (a > g.nv())][0]
        raise _lib.BoundsError(f"attempt to access vertex {bad} of a graph with {g.nv()} vertices")
    return (a - 1).astype(np.int32)


def betweenness_raw(g, src0: np.ndarray | None, endpoints: bool = False) -> np.ndarray:
    """Unscaled GPU accumulation over 0-based sources (None = all vertices)."""
    h = g.device_handle()
    out = np.empty(g.nv(), np.float64)
    if g.nv() == 0:
        return out
    src = None if src0 is None else np.ascontiguousarray(src0, np.int32)
    nsrc = 0 if src is None else len(src)
    _lib.check(_lib.lib().lgbc_betweenness(h.handle, _lib.ptr(src), nsrc, int(bool(endpoints)),
                                           _lib.ptr(out)))
    return out


def betweenness_centrality(g, vs=None, distmx=None, *, normalize: bool = True,
                           endpoints: bool = False, rng=None) -> np.ndarray:
    """Drop-in for LightGraphs.betweenness_centrality (betweenness.jl:46-78).

    ``vs`` is a collection of 1-based vertices (default: all), or an integer k
    for the sampled variant, which draws k distinct sources with ``sample``.
    Returns a float64 vector indexed by vertex - 1."""
    if _is_count(vs):
        vs = sample(g.vertices(), int(vs), rng=rng)
    _check_distmx(g, distmx)
    n = g.nv()
    if vs is None:
        k = n
        raw = betweenness_raw(g, None, endpoints)
    else:
        src0 = _sources0(g, vs)
        k = len(src0)
        raw = betweenness_raw(g, src0, endpoints)
    _rescale_(raw, n, normalize, g.is_directed(), k)
    return raw


def betweenness_centrality_many(graphs, *, normalize: bool = True,
                                endpoints: bool = False) -> list:
    """Exact betweenness_centrality(g) for every undirected graph in `graphs`,
    computed in one library call (lgbc_betweenness_many): graphs of similar
    size run together as disjoint unions, one lane per source index.
    Returns one float64 vector per graph, each rescaled with _rescale!."""
    graphs = list(graphs)
    if not graphs:
        return []
    for g in graphs:
        if g.is_directed():
            raise _lib.MethodError("betweenness_centrality_many covers undirected graphs")
    ns = np.array([g.nv() for g in graphs], np.int64)
    rps, cis = zip(*(g.csr() for g in graphs))
    rp_off = np.concatenate([[0], np.cumsum([len(r) for r in rps])[:-1]]).astype(np.int64)
    ci_off = np.concatenate([[0], np.cumsum([len(c) for c in cis])[:-1]]).astype(np.int64)
    rowptr = np.ascontiguousarray(np.concatenate(rps), np.int64)
    colidx = np.ascontiguousarray(np.concatenate(cis) if sum(len(c) for c in cis)
                                  else np.zeros(1, np.int32), np.int32)
    out = np.empty(int(ns.sum()), np.float64)
    _lib.check(_lib.lib().lgbc_betweenness_many(len(graphs), _lib.ptr(ns), _lib.ptr(rp_off),
                                                _lib.ptr(ci_off), _lib.ptr(rowptr), _lib.ptr(colidx),
                                                int(bool(endpoints)), _lib.ptr(out)))
    res, o = [], 0
    for g, n in zip(graphs, ns):
        v = out[o:o + n].copy()
        _rescale_(v, int(n), normalize, False, int(n))
        res.append(v)
        o += n
    return res


def stress_centrality(g, vs=None, *, rng=None) -> np.ndarray:
    """Drop-in for LightGraphs.stress_centrality (src/centrality/stress.jl:33-49):
    ``vs`` a collection of 1-based vertices (default all) or an integer k for
    ``sample(vertices(g), k)``.  Returns the Int64 stress vector (vertex - 1),
    with the reference's wrapping Int64 arithmetic."""
    if _is_count(vs):
        vs = sample(g.vertices(), int(vs), rng=rng)
    n = g.nv()
    out = np.zeros(n, np.int64)
    if n == 0:
        return out
    src = None if vs is None else np.ascontiguousarray(_sources0(g, vs), np.int32)
    nsrc = 0 if src is None else len(src)
    _lib.check(_lib.lib().lgbc_stress(g.device_handle().handle, _lib.ptr(src), nsrc,
                                      _lib.ptr(out)))
    return out
