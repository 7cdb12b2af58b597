"""The C-ABI library loads and exports every symbol the headers declare.
No GPU is needed: only calls that fail before touching a device are made."""
import ctypes
import os
import re

import pytest

import lgbc
from lgbc import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for h in sorted(os.listdir(inc)):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(inc, h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(lgbc_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for required in ("lgbc_graph_create", "lgbc_graph_destroy", "lgbc_gdistances",
                     "lgbc_gdistances_batch", "lgbc_betweenness", "lgbc_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol():
    lib = _lib.lib()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_errors_without_gpu():
    lib = _lib.lib()
    assert lib.lgbc_version().decode().startswith("lgbc")
    # argument errors are reported before any device work
    h = ctypes.c_void_p()
    rc = lib.lgbc_graph_create(ctypes.byref(h), -1, 0, None, None, None, None, 0)
    assert rc == _lib.LGBC_EINVAL and "negative" in _lib.last_error()
    rc = lib.lgbc_graph_create(None, 1, 0, None, None, None, None, 0)
    assert rc == _lib.LGBC_EINVAL
    assert lib.lgbc_betweenness(None, None, 0, 0, None) == _lib.LGBC_EINVAL
    assert lib.lgbc_gdistances(None, None, 0, None) == _lib.LGBC_EINVAL
    assert lib.lgbc_graph_destroy(None) == _lib.LGBC_OK


def test_no_cpu_fallback_without_gpu():
    lib = _lib.lib()
    if lib.lgbc_device_count() > 0:
        pytest.skip("a GPU is present")
    g = lgbc.SimpleGraph.from_edges(3, [(1, 2), (2, 3)])
    with pytest.raises(lgbc.LGBCError) as ei:
        lgbc.betweenness_centrality(g)
    assert "CUDA" in str(ei.value) or "device" in str(ei.value)
