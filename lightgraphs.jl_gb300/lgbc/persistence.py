"""Reader for LightGraphs' LG text format (plain or gzip-compressed).

Reference: src/persistence/lg.jl:1-80 (header ``nv,ne,{d|u},name[,ver,dtype,code]``
followed by ``src,dst`` lines, 1-based) and the gzip magic check of
src/persistence/common.jl:41-58.  Only the first graph of a file is read.
"""
from __future__ import annotations

import gzip

import numpy as np

from .graphs import SimpleDiGraph, SimpleGraph


def _open(path: str):
    with open(path, "rb") as f:
        magic = f.read(2)
    if magic == b"\x1f\x8b":
        return gzip.open(path, "rt")
    return open(path, "rt")


def loadgraph(path: str, eltype=np.int64):
    """loadgraph(path) for an LG file: returns SimpleGraph or SimpleDiGraph."""
    with _open(path) as f:
        header = f.readline()
        parts = [p.strip() for p in header.split(",")]
        n, m = int(parts[0]), int(parts[1])
        directed = parts[2] != "u"
        src, dst = [], []
        for _ in range(m):
            line = f.readline().strip()
            if not line:
                continue
            a, b = line.split(",")
            src.append(int(a) - 1)
            dst.append(int(b) - 1)
    cls = SimpleDiGraph if directed else SimpleGraph
    return cls.from_edge_arrays(n, np.asarray(src, np.int64), np.asarray(dst, np.int64), eltype)
