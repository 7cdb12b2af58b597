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


def _struct_fields(header_text, name):
    """(type, field) pairs of `typedef struct name { ... } name;` in a header."""
    text = re.sub(r"/\*.*?\*/", "", header_text, flags=re.S)
    m = re.search(r"typedef\s+struct\s+" + name + r"\s*\{(.*?)\}\s*" + name + ";", text, flags=re.S)
    assert m, name
    return [tuple(f.split()) for f in (x.strip() for x in m.group(1).split(";")) if f]


def test_tuning_struct_matches_header():
    # the Python mirror of lgbc_tuning must have the header's fields, in order,
    # with the same C types, so that lgbc_get_tuning / lgbc_set_tuning agree
    text = open(os.path.join(ROOT, "include", "lgbc.h")).read()
    fields = _struct_fields(text, "lgbc_tuning")
    ctypes_of = {"double": ctypes.c_double, "int32_t": ctypes.c_int32}
    assert [f for _, f in fields] == [n for n, _ in _lib.LgbcTuning._fields_]
    assert [ctypes_of[t] for t, _ in fields] == [c for _, c in _lib.LgbcTuning._fields_]
    assert "hub_order" in dict(_lib.LgbcTuning._fields_)


def test_bench_bytes_model():
    # the roofline numerator of the default workload (R-MAT 20, 2,549 active
    # sources): 20 batches of 128 (or 40 of 64) CSR passes + 32 n bytes per source
    import sys
    sys.path.insert(0, ROOT)
    import bench
    n, nnz, k = 1 << 20, 31401246, 2549
    assert bench.bc_algorithmic_bytes(n, nnz, k, 128) == 20 * (8 * nnz + 32 * n + 16) + 32 * n * k
    assert bench.bc_algorithmic_bytes(n, nnz, k, 128) == 91225535488
    assert bench.bc_algorithmic_bytes(n, nnz, k, 64) == 40 * (8 * nnz + 32 * n + 16) + 32 * n * k
