"""ctypes loader for the CPU oracle (``lg_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: the oracle is the checker for the CUDA library and
the timed CPU baseline.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline / reference arm import this module; the product
package never does.

The oracle restates LightGraphs.jl v1.3.5 (paths relative to that project):
  * ``gdistances``        -- src/traversals/bfs.jl:95-124,141
  * ``dijkstra``          -- src/shortestpaths/dijkstra.jl:59-144 (unit weights)
  * ``betweenness_raw``   -- src/centrality/betweenness.jl:46-134 before
                             ``_rescale!``; Parallel threaded variant
                             src/Parallel/centrality/betweenness.jl:42-72
  * ``rescale``           -- src/centrality/betweenness.jl:136-160
  * ``closeness``, ``radiality``, ``eccentricity``
                          -- src/centrality/closeness.jl:33-55,
                             src/centrality/radiality.jl:36-49, src/distance.jl:73-79
  * ``core_number``       -- src/degeneracy.jl:38-80
  * ``stress``            -- src/centrality/stress.jl:33-77
  * ``bfs_parents``, ``has_path`` -- src/traversals/bfs.jl:40-66, :150-172
  * ``gdistances_many``   -- gdistances per source, one source per host thread
Parity is pinned against the reference's golden vectors (tests/golden/).

The shared object also carries the seeded graph generators of the workloads
(``rmat``, ``erdos_renyi_nm``, ``barabasi_albert``): the library's own host
source lightgraphs.jl_gb300/csrc/generators.cpp compiled in here as well, so
that the CPU arm of bench.py builds the same graphs without mapping the CUDA
library.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "liblgoracle.so")
_SRC = os.path.join(_HERE, "lg_oracle.cpp")
_ROOT = os.path.dirname(_HERE)
_GEN = os.path.join(_ROOT, "lightgraphs.jl_gb300", "csrc", "generators.cpp")
_INC = os.path.join(_ROOT, "include")
_lock = threading.Lock()
_lib = None

UNREACHED32 = np.iinfo(np.int32).max
UNREACHED64 = np.iinfo(np.int64).max


def build(force: bool = False) -> str:
    """Compile the oracle into ``oracle/_build/liblgoracle.so`` (g++, -O3)."""
    os.makedirs(_BUILD, exist_ok=True)
    srcs = [_SRC, _GEN, os.path.join(_INC, "lgbc_gen.h")]
    if (not force and os.path.exists(_SO)
            and os.path.getmtime(_SO) >= max(os.path.getmtime(p) for p in srcs)):
        return _SO
    tmp = _SO + f".tmp{os.getpid()}"
    cmd = ["g++", "-O3", "-std=c++17", "-shared", "-fPIC", "-pthread", "-I", _INC,
           _SRC, _GEN, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _SO)
    return _SO


def _load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        build()
        lib = ctypes.CDLL(_SO)
        i64, i32, dbl = ctypes.c_int64, ctypes.c_int32, ctypes.c_double
        p = ctypes.c_void_p
        lib.orc_gdistances.argtypes = [i64, p, p, p, i64, p]
        lib.orc_gdistances.restype = ctypes.c_int
        lib.orc_gdistances_many.argtypes = [i64, p, p, p, i64, ctypes.c_int, p]
        lib.orc_gdistances_many.restype = ctypes.c_int
        P = ctypes.POINTER(_Csr)
        lib.lgbc_gen_rmat.argtypes = [ctypes.c_int, ctypes.c_int, dbl, dbl, dbl,
                                      ctypes.c_uint64, ctypes.c_int, P]
        lib.lgbc_gen_rmat.restype = ctypes.c_int
        lib.lgbc_gen_erdos_renyi.argtypes = [i64, i64, ctypes.c_uint64, ctypes.c_int, P]
        lib.lgbc_gen_erdos_renyi.restype = ctypes.c_int
        lib.lgbc_gen_barabasi_albert.argtypes = [i64, ctypes.c_int, ctypes.c_uint64, P]
        lib.lgbc_gen_barabasi_albert.restype = ctypes.c_int
        lib.lgbc_csr_free.argtypes = [P]
        lib.lgbc_csr_free.restype = None
        lib.orc_dijkstra.argtypes = [i64, p, p, i32, p, p, p, p, p, i64]
        lib.orc_dijkstra.restype = i64
        lib.orc_betweenness.argtypes = [i64, p, p, p, p, ctypes.c_int, p, i64,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, p]
        lib.orc_betweenness.restype = ctypes.c_int
        lib.orc_rescale.argtypes = [p, i64, ctypes.c_int, ctypes.c_int, i64]
        lib.orc_rescale.restype = None
        lib.orc_dependency.argtypes = [i64, p, p, p, p, ctypes.c_int, p, p, i64, p, p]
        lib.orc_dependency.restype = ctypes.c_int
        lib.orc_stress.argtypes = [i64, p, p, p, p, ctypes.c_int, p, i64, p]
        lib.orc_stress.restype = ctypes.c_int
        lib.orc_core_number.argtypes = [i64, p, p, p, p, ctypes.c_int, p]
        lib.orc_core_number.restype = ctypes.c_int
        _lib = lib
        return lib


class _Csr(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("nnz", ctypes.c_int64), ("m", ctypes.c_int64),
                ("directed", ctypes.c_int), ("rowptr", ctypes.POINTER(ctypes.c_int64)),
                ("colidx", ctypes.POINTER(ctypes.c_int32)),
                ("in_rowptr", ctypes.POINTER(ctypes.c_int64)),
                ("in_colidx", ctypes.POINTER(ctypes.c_int32))]


class CsrGraph:
    """A generated graph as plain arrays: rowptr / colidx (out-lists), the
    in-lists of a digraph, m (edges counted once, or arcs)."""

    def __init__(self, c: _Csr):
        n, nnz = int(c.n), int(c.nnz)
        self.n, self.m, self.directed = n, int(c.m), bool(c.directed)
        self.rowptr = np.ctypeslib.as_array(c.rowptr, shape=(n + 1,)).copy()
        self.colidx = (np.ctypeslib.as_array(c.colidx, shape=(nnz,)).copy() if nnz
                       else np.zeros(0, np.int32))
        self.in_rowptr = self.in_colidx = None
        if self.directed:
            self.in_rowptr = np.ctypeslib.as_array(c.in_rowptr, shape=(n + 1,)).copy()
            self.in_colidx = (np.ctypeslib.as_array(c.in_colidx, shape=(nnz,)).copy() if nnz
                              else np.zeros(0, np.int32))

    def nv(self):
        return self.n

    def ne(self):
        return self.m

    def is_directed(self):
        return self.directed

    def csr(self):
        return self.rowptr, self.colidx

    def in_csr(self):
        return (self.in_rowptr, self.in_colidx) if self.directed else (self.rowptr, self.colidx)

    def degrees(self):
        d = np.diff(self.rowptr)
        return d + np.diff(self.in_rowptr) if self.directed else d


def _generated(rc, c):
    lib = _load()
    if rc != 0:
        raise ValueError("generator parameters out of range")
    g = CsrGraph(c)
    lib.lgbc_csr_free(ctypes.byref(c))
    return g


def rmat(scale, edgefactor=16, a=0.57, b=0.19, c=0.19, *, seed=1, directed=False) -> CsrGraph:
    """The library's R-MAT generator (same source, same seeds, same graph)."""
    out = _Csr()
    rc = _load().lgbc_gen_rmat(int(scale), int(edgefactor), float(a), float(b), float(c),
                               int(seed) & (2**64 - 1), int(bool(directed)), ctypes.byref(out))
    return _generated(rc, out)


def erdos_renyi_nm(n, m, *, seed=1, directed=False) -> CsrGraph:
    out = _Csr()
    rc = _load().lgbc_gen_erdos_renyi(int(n), int(m), int(seed) & (2**64 - 1),
                                      int(bool(directed)), ctypes.byref(out))
    return _generated(rc, out)


def barabasi_albert(n, k, *, seed=1) -> CsrGraph:
    out = _Csr()
    rc = _load().lgbc_gen_barabasi_albert(int(n), int(k), int(seed) & (2**64 - 1),
                                          ctypes.byref(out))
    return _generated(rc, out)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _csr(rowptr, colidx):
    return (np.ascontiguousarray(rowptr, dtype=np.int64),
            np.ascontiguousarray(colidx, dtype=np.int32))


def gdistances(rowptr, colidx, sources) -> np.ndarray:
    """Multi-source level-synchronous BFS; INT32_MAX marks unreached."""
    lib = _load()
    rowptr, colidx = _csr(rowptr, colidx)
    n = len(rowptr) - 1
    src = np.ascontiguousarray(np.atleast_1d(np.asarray(sources, dtype=np.int32)))
    dist = np.empty(n, dtype=np.int32)
    rc = lib.orc_gdistances(n, _ptr(rowptr), _ptr(colidx), _ptr(src), len(src), _ptr(dist))
    if rc != 0:
        raise ValueError("oracle gdistances: bad source")
    return dist


def gdistances_many(rowptr, colidx, sources, nthreads=1) -> np.ndarray:
    """One single-source gdistances per source, (len, n) int32, one source
    per host thread."""
    lib = _load()
    rowptr, colidx = _csr(rowptr, colidx)
    n = len(rowptr) - 1
    src = np.ascontiguousarray(np.atleast_1d(np.asarray(sources, dtype=np.int32)))
    dist = np.empty((len(src), n), dtype=np.int32)
    rc = lib.orc_gdistances_many(n, _ptr(rowptr), _ptr(colidx), _ptr(src), len(src),
                                 int(nthreads), _ptr(dist))
    if rc != 0:
        raise ValueError("oracle gdistances: bad source")
    return dist


def dijkstra(rowptr, colidx, s):
    """Unit-weight Dijkstra with all paths: (dists, pathcounts, preds, closest)."""
    lib = _load()
    rowptr, colidx = _csr(rowptr, colidx)
    n = len(rowptr) - 1
    dists = np.empty(n, np.int64)
    pc = np.empty(n, np.float64)
    closest = np.empty(n, np.int32)
    poff = np.empty(n + 1, np.int64)
    cap = max(1, len(colidx))
    pred = np.empty(cap, np.int32)
    tot = lib.orc_dijkstra(n, _ptr(rowptr), _ptr(colidx), int(s), _ptr(dists), _ptr(pc),
                           _ptr(closest), _ptr(poff), _ptr(pred), cap)
    if tot < 0:
        raise ValueError("oracle dijkstra failed")
    preds = [pred[poff[v]:poff[v + 1]].tolist() for v in range(n)]
    return dists, pc, preds, closest


def betweenness_raw(rowptr, colidx, sources, *, directed=False, in_rowptr=None,
                    in_colidx=None, endpoints=False, mode="fast", nthreads=1) -> np.ndarray:
    """Unscaled BC over an explicit source list (degree-0 sources skipped)."""
    lib = _load()
    rowptr, colidx = _csr(rowptr, colidx)
    n = len(rowptr) - 1
    if directed:
        in_rowptr, in_colidx = _csr(in_rowptr, in_colidx)
    else:
        in_rowptr = in_colidx = None
    src = np.ascontiguousarray(np.asarray(sources, dtype=np.int32).ravel())
    out = np.empty(n, np.float64)
    rc = lib.orc_betweenness(n, _ptr(rowptr), _ptr(colidx), _ptr(in_rowptr), _ptr(in_colidx),
                             int(bool(directed)), _ptr(src), len(src), int(bool(endpoints)),
                             0 if mode == "faithful" else 1, int(nthreads), _ptr(out))
    if rc != 0:
        raise ValueError("oracle betweenness: bad arguments")
    return out


def rescale(bc, n, normalize, directed, k) -> np.ndarray:
    """_rescale! on a copy (src/centrality/betweenness.jl:136-160)."""
    lib = _load()
    out = np.ascontiguousarray(bc, dtype=np.float64).copy()
    lib.orc_rescale(_ptr(out), int(n), int(bool(normalize)), int(bool(directed)), int(k))
    return out


def betweenness_centrality(rowptr, colidx, sources=None, *, directed=False, in_rowptr=None,
                           in_colidx=None, normalize=True, endpoints=False, mode="fast",
                           nthreads=1) -> np.ndarray:
    """The full reference result: raw accumulation followed by ``_rescale!``."""
    n = len(rowptr) - 1
    if sources is None:
        sources = np.arange(n, dtype=np.int32)
    src = np.asarray(sources, dtype=np.int32).ravel()
    raw = betweenness_raw(rowptr, colidx, src, directed=directed, in_rowptr=in_rowptr,
                          in_colidx=in_colidx, endpoints=endpoints, mode=mode,
                          nthreads=nthreads)
    return rescale(raw, n, normalize, directed, len(src))


def dependency(rowptr, colidx, sources, weights=None, *, directed=False, in_rowptr=None,
               in_colidx=None):
    """(mass per source, weighted accumulation sum_i w_i delta_{s_i})."""
    lib = _load()
    rowptr, colidx = _csr(rowptr, colidx)
    n = len(rowptr) - 1
    if directed:
        in_rowptr, in_colidx = _csr(in_rowptr, in_colidx)
    else:
        in_rowptr = in_colidx = None
    src = np.ascontiguousarray(np.asarray(sources, dtype=np.int32).ravel())
    w = None if weights is None else np.ascontiguousarray(weights, np.float64)
    mass = np.empty(len(src), np.float64)
    bcw = np.empty(n, np.float64)
    rc = lib.orc_dependency(n, _ptr(rowptr), _ptr(colidx), _ptr(in_rowptr), _ptr(in_colidx),
                            int(bool(directed)), _ptr(src), _ptr(w), len(src), _ptr(mass), _ptr(bcw))
    if rc != 0:
        raise ValueError("oracle dependency: bad arguments")
    return mass, bcw


def core_number(rowptr, colidx, *, directed=False, in_rowptr=None, in_colidx=None) -> np.ndarray:
    """core_number(g) (src/degeneracy.jl:38-96)."""
    lib = _load()
    rowptr, colidx = _csr(rowptr, colidx)
    n = len(rowptr) - 1
    if directed:
        in_rowptr, in_colidx = _csr(in_rowptr, in_colidx)
    else:
        in_rowptr = in_colidx = None
    out = np.empty(n, np.int32)
    if lib.orc_core_number(n, _ptr(rowptr), _ptr(colidx), _ptr(in_rowptr), _ptr(in_colidx),
                           int(bool(directed)), _ptr(out)) != 0:
        raise ValueError("core_number: graph must not have self-loops")
    return out


def features(rowptr, colidx) -> np.ndarray:
    """The four source features of the learned proposal, per vertex:
    log(1+deg), log(1+core number), mean log(1+deg) of the neighbours, and
    log(1 + sum of the neighbours' degrees) (a two-hop count estimate)."""
    rowptr, colidx = _csr(rowptr, colidx)
    n = len(rowptr) - 1
    deg = np.diff(rowptr).astype(np.float64)
    ld = np.log1p(deg)
    src = np.repeat(np.arange(n), np.diff(rowptr))
    s_ld = np.bincount(src, weights=ld[colidx], minlength=n)
    s_d = np.bincount(src, weights=deg[colidx], minlength=n)
    f = np.empty((n, 4), np.float64)
    f[:, 0] = ld
    f[:, 1] = np.log1p(core_number(rowptr, colidx).astype(np.float64))
    f[:, 2] = np.where(deg > 0, s_ld / np.maximum(deg, 1.0), 0.0)
    f[:, 3] = np.log1p(s_d)
    return f


_TYPEMAX = np.iinfo(np.int64).max


def _dists64(rowptr, colidx, s):
    """dijkstra_shortest_paths(g, s).dists with unit weights: Int64, typemax unreached."""
    d = gdistances(rowptr, colidx, [s]).astype(np.int64)
    d[d == UNREACHED32] = _TYPEMAX
    return d


def closeness(rowptr, colidx, degrees, normalize=True) -> np.ndarray:
    """closeness_centrality (src/centrality/closeness.jl:33-55); degrees as
    degree(g, v) (in + out for a digraph)."""
    n = len(rowptr) - 1
    out = np.zeros(n)
    for u in range(n):
        if degrees[u] == 0:
            continue
        d = _dists64(rowptr, colidx, u)
        delta = d[d != _TYPEMAX]
        sigma = int(delta.sum())
        l = len(delta) - 1
        if sigma > 0:
            out[u] = l / sigma
            if normalize:
                out[u] *= l / (n - 1)
    return out


def radiality(rowptr, colidx) -> np.ndarray:
    """radiality_centrality (src/centrality/radiality.jl:36-49), Int64
    sums wrapping as Julia's do."""
    n = len(rowptr) - 1
    meandists = np.zeros(n)
    dmtr = 0.0
    with np.errstate(over="ignore"):
        for v in range(n):
            d = _dists64(rowptr, colidx, v)
            dmtr = max(dmtr, float(d.max()))
            meandists[v] = float(d.sum(dtype=np.int64)) / (n - 1)
    meandists = (dmtr + 1) - meandists
    return meandists / dmtr


def eccentricity(rowptr, colidx, vs=None) -> np.ndarray:
    """eccentricity(g, vs) (src/distance.jl:73-84): Int64, typemax if unreachable."""
    n = len(rowptr) - 1
    vs = range(n) if vs is None else vs
    return np.array([int(_dists64(rowptr, colidx, v).max()) for v in vs], np.int64)


def stress(rowptr, colidx, sources=None, *, directed=False, in_rowptr=None, in_colidx=None):
    """stress_centrality(g, vs) (src/centrality/stress.jl:33-77), Int64."""
    lib = _load()
    rowptr, colidx = _csr(rowptr, colidx)
    n = len(rowptr) - 1
    if directed:
        in_rowptr, in_colidx = _csr(in_rowptr, in_colidx)
    else:
        in_rowptr = in_colidx = None
    src = np.arange(n, dtype=np.int32) if sources is None else \
        np.ascontiguousarray(np.asarray(sources, dtype=np.int32).ravel())
    out = np.empty(n, np.int64)
    if lib.orc_stress(n, _ptr(rowptr), _ptr(colidx), _ptr(in_rowptr), _ptr(in_colidx),
                      int(bool(directed)), _ptr(src), len(src), _ptr(out)) != 0:
        raise ValueError("oracle stress: bad arguments")
    return out


def bfs_parents(rowptr, colidx, s: int) -> np.ndarray:
    """_bfs_parents(g, s, neighborfn) (src/traversals/bfs.jl:40-66) over the
    given CSR (the out-lists for :out, the in-lists for :in); 0-based ids,
    -1 where unreached.  Pure Python, for small graphs."""
    n = len(rowptr) - 1
    visited = np.zeros(n, bool)
    parents = np.full(n, -1, np.int64)
    cur = [s]
    visited[s] = True
    parents[s] = s
    while cur:
        nxt = []
        for v in cur:
            for i in colidx[rowptr[v]:rowptr[v + 1]].tolist():
                if not visited[i]:
                    nxt.append(i)
                    parents[i] = v
                    visited[i] = True
        cur = sorted(nxt)
    return parents


def has_path(rowptr, colidx, u: int, v: int, exclude=()) -> bool:
    """has_path(g, u, v; exclude_vertices) (src/traversals/bfs.jl:150-172), 0-based."""
    n = len(rowptr) - 1
    seen = np.zeros(n, bool)
    for x in exclude:
        seen[x] = True
    if seen[u] or seen[v]:
        return False
    if u == v:
        return True
    q = [u]
    seen[u] = True
    while q:
        x = q.pop(0)
        for w in colidx[rowptr[x]:rowptr[x + 1]].tolist():
            if w == v:
                return True
            if not seen[w]:
                q.append(w)
                seen[w] = True
    return False
