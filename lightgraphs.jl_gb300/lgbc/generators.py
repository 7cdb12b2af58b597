"""Seeded graph generators (host C++ in liblgbc.so, include/lgbc_gen.h).

They follow the semantics of LightGraphs' generators
(src/SimpleGraphs/generators/randgraphs.jl) with a SplitMix64 stream, so the
graphs are distributionally, not bit-for-bit, those of the reference.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .graphs import SimpleDiGraph, SimpleGraph


class _Csr(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("nnz", ctypes.c_int64), ("m", ctypes.c_int64),
                ("directed", ctypes.c_int), ("rowptr", ctypes.POINTER(ctypes.c_int64)),
                ("colidx", ctypes.POINTER(ctypes.c_int32)),
                ("in_rowptr", ctypes.POINTER(ctypes.c_int64)),
                ("in_colidx", ctypes.POINTER(ctypes.c_int32))]


_declared = False


def _gen():
    global _declared
    lib = _lib.lib()
    if not _declared:
        P = ctypes.POINTER(_Csr)
        lib.lgbc_gen_rmat.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_uint64, ctypes.c_int, P]
        lib.lgbc_gen_rmat.restype = ctypes.c_int
        lib.lgbc_gen_erdos_renyi.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_uint64,
                                             ctypes.c_int, P]
        lib.lgbc_gen_erdos_renyi.restype = ctypes.c_int
        lib.lgbc_gen_barabasi_albert.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_uint64, P]
        lib.lgbc_gen_barabasi_albert.restype = ctypes.c_int
        lib.lgbc_csr_free.argtypes = [P]
        lib.lgbc_csr_free.restype = None
        _declared = True
    return lib


def _adopt(c: _Csr, eltype):
    n, nnz = int(c.n), int(c.nnz)
    rp = np.ctypeslib.as_array(c.rowptr, shape=(n + 1,)).copy()
    ci = (np.ctypeslib.as_array(c.colidx, shape=(nnz,)).copy() if nnz
          else np.zeros(0, np.int32))
    if c.directed:
        irp = np.ctypeslib.as_array(c.in_rowptr, shape=(n + 1,)).copy()
        ici = (np.ctypeslib.as_array(c.in_colidx, shape=(nnz,)).copy() if nnz
               else np.zeros(0, np.int32))
        g = SimpleDiGraph.from_csr(rp, ci, irp, ici, eltype=eltype)
    else:
        g = SimpleGraph.from_csr(rp, ci, eltype=eltype)
    _gen().lgbc_csr_free(ctypes.byref(c))
    return g


def rmat(scale: int, edgefactor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
         *, seed: int = 1, directed: bool = False, eltype=np.int32):
    """R-MAT / Kronecker graph (kronecker, randgraphs.jl:1126-1152) with
    self-loops and duplicates removed; undirected unless ``directed``."""
    out = _Csr()
    rc = _gen().lgbc_gen_rmat(int(scale), int(edgefactor), float(a), float(b), float(c),
                              int(seed) & (2**64 - 1), int(bool(directed)), ctypes.byref(out))
    if rc != 0:
        raise _lib.ArgumentError("invalid R-MAT parameters")
    return _adopt(out, eltype)


def erdos_renyi_nm(n: int, m: int, *, seed: int = 1, directed: bool = False, eltype=np.int64):
    """G(n, m) as SimpleGraph(nv, ne; seed) (randgraphs.jl:25-40)."""
    out = _Csr()
    rc = _gen().lgbc_gen_erdos_renyi(int(n), int(m), int(seed) & (2**64 - 1),
                                     int(bool(directed)), ctypes.byref(out))
    if rc != 0:
        raise _lib.ArgumentError("invalid G(n, m) parameters (m must be <= 2/3 of the maximum)")
    return _adopt(out, eltype)


def barabasi_albert(n: int, k: int, *, seed: int = 1, eltype=np.int64):
    """barabasi_albert(n, k; seed) (randgraphs.jl:391-392, 449-512)."""
    out = _Csr()
    rc = _gen().lgbc_gen_barabasi_albert(int(n), int(k), int(seed) & (2**64 - 1),
                                         ctypes.byref(out))
    if rc != 0:
        raise _lib.ArgumentError("barabasi_albert requires 1 <= k <= n")
    return _adopt(out, eltype)
