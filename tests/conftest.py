"""Shared test setup: import paths, the ``gpu`` marker and fixture loaders."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "lightgraphs.jl_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


def golden_path(name: str) -> str:
    return os.path.join(GOLDEN, name)


@pytest.fixture(scope="session")
def known():
    with open(golden_path("known_answers.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_graph():
    import lgbc
    return lgbc.loadgraph(golden_path("graph-50-500.lg"))


@pytest.fixture(scope="session")
def golden_bc():
    return np.loadtxt(golden_path("graph-50-500-bc.txt"))


def make_graph(case):
    """SimpleGraph / SimpleDiGraph from a known-answer JSON entry (1-based edges)."""
    import lgbc
    cls = lgbc.SimpleDiGraph if case["directed"] else lgbc.SimpleGraph
    return cls.from_edges(case["n"], case["edges"])


def csr_args(g):
    """Keyword arguments for the oracle from a graph."""
    rp, ci = g.csr()
    kw = dict(directed=g.is_directed())
    if g.is_directed():
        irp, ici = g.in_csr()
        kw.update(in_rowptr=irp, in_colidx=ici)
    return rp, ci, kw
