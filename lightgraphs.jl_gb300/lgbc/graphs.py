"""SimpleGraph / SimpleDiGraph mirrors with CSR storage, plus the device handle.

LightGraphs stores a graph as ``fadjlist::Vector{Vector{T}}`` (and
``badjlist`` for digraphs), each neighbour list sorted ascending and free of
duplicates (src/SimpleGraphs/simplegraph.jl:8-16, :445-461;
simpledigraph.jl:8-21, :414-429).  These classes keep exactly that content
flattened to a 0-based CSR -- ``rowptr`` (int64, n+1) and ``colidx`` (int32)
-- which is also the layout the C ABI uploads.  Vertex ids in the public
methods are 1-based, as in Julia.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _csr_from_pairs(n: int, src: np.ndarray, dst: np.ndarray):
    """Sorted, de-duplicated CSR of the (src, dst) pairs (0-based)."""
    if len(src) == 0:
        return np.zeros(n + 1, np.int64), np.zeros(0, np.int32)
    key = np.unique(src.astype(np.int64) * n + dst.astype(np.int64))
    s = key // n
    d = (key % n).astype(np.int32)
    counts = np.bincount(s, minlength=n)
    rowptr = np.zeros(n + 1, np.int64)
    np.cumsum(counts, out=rowptr[1:])
    return rowptr, d


class _GraphBase:
    directed = False

    def __init__(self, n: int = 0, eltype=np.int64):
        if n < 0:
            raise _lib.ArgumentError("number of vertices must be non-negative")
        self._n = int(n)
        self.eltype = np.dtype(eltype)
        self._pending: list[tuple[int, int]] = []
        self._src = np.zeros(0, np.int64)
        self._dst = np.zeros(0, np.int64)
        self._csr = None
        self._in_csr = None
        self._handle = None

    # -- construction ------------------------------------------------------
    @classmethod
    def from_edge_arrays(cls, n: int, src0, dst0, eltype=np.int64):
        """Graph from 0-based endpoint arrays (duplicates are dropped, as
        repeated add_edge! calls would)."""
        g = cls(n, eltype)
        g._src = np.asarray(src0, np.int64).ravel()
        g._dst = np.asarray(dst0, np.int64).ravel()
        if len(g._src) and (g._src.min() < 0 or g._dst.min() < 0 or
                            g._src.max() >= n or g._dst.max() >= n):
            raise _lib.BoundsError("edge endpoint outside 0:n-1")
        return g

    @classmethod
    def from_edges(cls, n: int, edges, eltype=np.int64):
        """Graph from 1-based (u, v) pairs."""
        e = np.asarray(list(edges), np.int64).reshape(-1, 2)
        return cls.from_edge_arrays(n, e[:, 0] - 1, e[:, 1] - 1, eltype)

    @classmethod
    def from_csr(cls, rowptr, colidx, in_rowptr=None, in_colidx=None, eltype=np.int64):
        """Adopt an already sorted, de-duplicated CSR (0-based)."""
        rowptr = np.ascontiguousarray(rowptr, np.int64)
        colidx = np.ascontiguousarray(colidx, np.int32)
        n = len(rowptr) - 1
        g = cls(n, eltype)
        g._csr = (rowptr, colidx)
        if cls.directed:
            if in_rowptr is None:
                in_rowptr, in_colidx = _transpose(n, rowptr, colidx)
            g._in_csr = (np.ascontiguousarray(in_rowptr, np.int64),
                         np.ascontiguousarray(in_colidx, np.int32))
        return g

    def add_edge(self, u: int, v: int) -> bool:
        """add_edge!(g, u, v) with 1-based ids (duplicates are ignored)."""
        if not (1 <= u <= self._n and 1 <= v <= self._n):
            return False
        self._materialise()
        self._pending.append((u - 1, v - 1))
        self._invalidate()
        return True

    def add_vertices(self, k: int) -> None:
        self._materialise()
        self._n += int(k)
        self._invalidate()

    # -- queries -----------------------------------------------------------
    def nv(self) -> int:
        return self._n

    def is_directed(self) -> bool:
        return self.directed

    def csr(self):
        """(rowptr int64[n+1], colidx int32[nnz]) of the out-neighbour lists."""
        if self._csr is None:
            self._build()
        return self._csr

    def in_csr(self):
        """CSR of the in-neighbour lists (badjlist); the same arrays for a graph."""
        if not self.directed:
            return self.csr()
        if self._in_csr is None:
            self._build()
        return self._in_csr

    def has_edge(self, u: int, v: int) -> bool:
        """has_edge(g, u, v) with 1-based ids (sorted out-list search)."""
        if not (1 <= u <= self._n and 1 <= v <= self._n):
            return False
        rp, ci = self.csr()
        row = ci[rp[u - 1]:rp[u]]
        i = int(np.searchsorted(row, v - 1))
        return i < len(row) and int(row[i]) == v - 1

    def outneighbors(self, v: int) -> np.ndarray:
        rp, ci = self.csr()
        return ci[rp[v - 1]:rp[v]].astype(np.int64) + 1

    def inneighbors(self, v: int) -> np.ndarray:
        rp, ci = self.in_csr()
        return ci[rp[v - 1]:rp[v]].astype(np.int64) + 1

    def vertices(self) -> range:
        return range(1, self._n + 1)

    # -- device handle -----------------------------------------------------
    def device_handle(self) -> "DeviceGraph":
        """The cached device-resident copy (re-uploaded after a mutation)."""
        if self._handle is None:
            self._handle = DeviceGraph(self)
        return self._handle

    # -- internals -----------------------------------------------------------
    def _invalidate(self) -> None:
        self._csr = None
        self._in_csr = None
        if self._handle is not None:
            self._handle.close()
            self._handle = None

    def _materialise(self) -> None:
        """Turn an adopted CSR back into edge arrays before a mutation."""
        if self._csr is not None and len(self._src) == 0 and not self._pending:
            rp, ci = self._csr
            self._src = np.repeat(np.arange(self._n, dtype=np.int64), np.diff(rp))
            self._dst = ci.astype(np.int64)

    def _pairs(self):
        src, dst = self._src, self._dst
        if self._pending:
            p = np.asarray(self._pending, np.int64)
            src = np.concatenate([src, p[:, 0]])
            dst = np.concatenate([dst, p[:, 1]])
            self._src, self._dst, self._pending = src, dst, []
        return src, dst


def _transpose(n, rowptr, colidx):
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(rowptr))
    return _csr_from_pairs(n, colidx.astype(np.int64), src)


class SimpleGraph(_GraphBase):
    """Undirected simple graph (src/SimpleGraphs/simplegraph.jl:8-16).  A
    self-loop is stored once in its vertex's list (simplegraph.jl:455)."""

    directed = False

    def _build(self):
        src, dst = self._pairs()
        a = np.concatenate([src, dst])
        b = np.concatenate([dst, src])
        self._csr = _csr_from_pairs(self._n, a, b)

    def ne(self) -> int:
        rp, ci = self.csr()
        loops = int(np.count_nonzero(np.repeat(np.arange(self._n), np.diff(rp)) == ci))
        return (len(ci) - loops) // 2 + loops

    def degree(self, v: int) -> int:
        """length(fadjlist[v]) (src/core.jl:67; a self-loop counts once)."""
        rp, _ = self.csr()
        return int(rp[v] - rp[v - 1])

    def degrees(self) -> np.ndarray:
        return np.diff(self.csr()[0])


class SimpleDiGraph(_GraphBase):
    """Directed simple graph with in-lists (src/SimpleGraphs/simpledigraph.jl:8-21)."""

    directed = True

    def _build(self):
        src, dst = self._pairs()
        self._csr = _csr_from_pairs(self._n, src, dst)
        self._in_csr = _csr_from_pairs(self._n, dst, src)

    def ne(self) -> int:
        return len(self.csr()[1])

    def degree(self, v: int) -> int:
        """indegree + outdegree (src/core.jl:66)."""
        rp, _ = self.csr()
        irp, _ = self.in_csr()
        return int(rp[v] - rp[v - 1] + irp[v] - irp[v - 1])

    def degrees(self) -> np.ndarray:
        return np.diff(self.csr()[0]) + np.diff(self.in_csr()[0])


def nv(g) -> int:
    return g.nv()


def ne(g) -> int:
    return g.ne()


def is_directed(g) -> bool:
    return g.is_directed()


def vertices(g) -> range:
    return g.vertices()


def degree(g, v: int) -> int:
    return g.degree(v)


class DefaultDistance:
    """Mirror of LightGraphs.DefaultDistance (src/distance.jl:8-21): an
    nv x nv matrix whose every entry is 1 -- the only weights the GPU path takes."""

    def __init__(self, nv: int):
        self.nv = int(nv)

    @property
    def shape(self):
        return (self.nv, self.nv)

    def __getitem__(self, ij):
        return 1


def weights(g) -> DefaultDistance:
    """weights(g) of a simple graph (src/core.jl:414)."""
    return DefaultDistance(g.nv())


class DeviceGraph:
    """A graph uploaded to the GPU through lgbc_graph_create."""

    @classmethod
    def adopt(cls, handle: ctypes.c_void_p, n: int, nnz: int, directed: bool) -> "DeviceGraph":
        """Wrap a handle the library already created (it is destroyed with the wrapper)."""
        d = cls.__new__(cls)
        d._h = handle
        d.n = n
        d.nnz = nnz
        d.directed = directed
        return d

    def __init__(self, g: _GraphBase):
        lib = _lib.lib()
        rp, ci = g.csr()
        irp, ici = (g.in_csr() if g.directed else (None, None))
        h = ctypes.c_void_p()
        _lib.check(lib.lgbc_graph_create(ctypes.byref(h), g.nv(), len(ci), _lib.ptr(rp),
                                         _lib.ptr(ci), _lib.ptr(irp), _lib.ptr(ici),
                                         int(g.directed)))
        self._h = h
        self.n = g.nv()
        self.nnz = len(ci)
        self.directed = g.directed

    @property
    def handle(self) -> ctypes.c_void_p:
        if self._h is None:
            raise _lib.LGBCError(_lib.LGBC_EINVAL, "device graph already closed")
        return self._h

    def stats(self) -> dict:
        s = _lib.LgbcStats()
        _lib.check(_lib.lib().lgbc_graph_stats(self.handle, ctypes.byref(s)))
        return s.as_dict()

    def tuning(self) -> _lib.LgbcTuning:
        t = _lib.LgbcTuning()
        _lib.check(_lib.lib().lgbc_get_tuning(self.handle, ctypes.byref(t)))
        return t

    def set_tuning(self, **kw) -> None:
        t = self.tuning()
        for k, v in kw.items():
            setattr(t, k, v)
        _lib.check(_lib.lib().lgbc_set_tuning(self.handle, ctypes.byref(t)))

    def tune(self, cache_path: str | None = None) -> dict:
        """Run the autotuner (lgbc_tune) and return the chosen settings."""
        path = None if cache_path is None else str(cache_path).encode()
        _lib.check(_lib.lib().lgbc_tune(self.handle, path))
        t = self.tuning()
        return {name: getattr(t, name) for name, _ in t._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            _lib.lib().lgbc_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def graph_from_edges(n: int, src0, dst0, *, directed: bool = False, eltype=np.int64):
    """SimpleGraph / SimpleDiGraph from 0-based endpoint arrays, with the CSR
    built on the GPU (lgbc_graph_create_from_edges: radix sort of the arcs,
    duplicates dropped, an undirected self-loop stored once -- the add_edge!
    semantics of src/SimpleGraphs/simplegraph.jl:445-461 and
    simpledigraph.jl:414-429).  The device copy stays attached to the graph."""
    src = np.ascontiguousarray(np.asarray(src0).ravel(), np.int64)
    dst = np.ascontiguousarray(np.asarray(dst0).ravel(), np.int64)
    if src.shape != dst.shape:
        raise _lib.ArgumentError("src and dst differ in length")
    if len(src) and (min(src.min(), dst.min()) < 0 or max(src.max(), dst.max()) >= n):
        raise _lib.BoundsError("edge endpoint outside 0:n-1")
    s32 = src.astype(np.int32)
    d32 = dst.astype(np.int32)
    lib = _lib.lib()
    h = ctypes.c_void_p()
    _lib.check(lib.lgbc_graph_create_from_edges(ctypes.byref(h), int(n), len(s32), _lib.ptr(s32),
                                                _lib.ptr(d32), int(bool(directed))))
    dev = DeviceGraph.adopt(h, int(n), 0, bool(directed))
    nn = ctypes.c_int64()
    nnz = ctypes.c_int64()
    _lib.check(lib.lgbc_graph_info(h, ctypes.byref(nn), ctypes.byref(nnz), None))
    dev.nnz = int(nnz.value)
    rp = np.empty(int(n) + 1, np.int64)
    ci = np.empty(max(int(nnz.value), 1), np.int32)
    irp = ici = None
    if directed:
        irp = np.empty(int(n) + 1, np.int64)
        ici = np.empty(max(int(nnz.value), 1), np.int32)
    _lib.check(lib.lgbc_graph_csr(h, _lib.ptr(rp), _lib.ptr(ci), _lib.ptr(irp), _lib.ptr(ici)))
    ci = ci[:int(nnz.value)]
    cls = SimpleDiGraph if directed else SimpleGraph
    if directed:
        g = cls.from_csr(rp, ci, irp, ici[:int(nnz.value)], eltype=eltype)
    else:
        g = cls.from_csr(rp, ci, eltype=eltype)
    g._handle = dev
    return g
