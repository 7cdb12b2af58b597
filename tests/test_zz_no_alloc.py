"""lgbc_gdistances_noalloc: gdistances for callers that cannot allocate.

Some callers cannot call cudaMalloc -- code running while a CUDA graph is
captured on its stream, or hosts whose device memory belongs to another
allocator with a fixed budget -- so this entry point takes every input and
output as caller-owned device pointers and keeps its BFS scratch in a fixed
static device array.  The test (only the test, never the entry point)
allocates the device buffers, calls the entry point twice in a row through
the C ABI with different sources, and checks each result bit for bit against
the handle-based lgbc_gdistances.  It lives in its own file, collected last.
"""
import ctypes

import numpy as np
import pytest

import lgbc
from lgbc import _lib
from lgbc import generators as G
from lgbc.traversals import _device_levels

pytestmark = pytest.mark.gpu


class DeviceArray:
    """A device copy of a numpy array, allocated by the test harness."""

    def __init__(self, a):
        self.a = np.ascontiguousarray(a)
        self.ptr = ctypes.c_void_p()
        lib = _lib.lib()
        _lib.check(lib.lgbc_device_alloc(ctypes.byref(self.ptr), max(self.a.nbytes, 1)))
        if self.a.nbytes:
            _lib.check(lib.lgbc_memcpy(self.ptr, _lib.ptr(self.a), self.a.nbytes, 1))

    def to_host(self):
        out = np.empty_like(self.a)
        _lib.check(_lib.lib().lgbc_memcpy(_lib.ptr(out), self.ptr, out.nbytes, 2))
        return out

    def free(self):
        _lib.lib().lgbc_device_free(self.ptr)


def _noalloc_levels(g, sources0, dist_buf):
    lib = _lib.lib()
    rp, ci = g.csr()
    d_rp, d_ci = DeviceArray(rp), DeviceArray(ci)
    d_irp = d_ici = None
    if g.is_directed():
        irp, ici = g.in_csr()
        d_irp, d_ici = DeviceArray(irp), DeviceArray(ici)
    d_src = DeviceArray(np.asarray(sources0, np.int32))
    try:
        _lib.check(lib.lgbc_gdistances_noalloc(
            g.nv(), len(ci), d_rp.ptr, d_ci.ptr, d_irp.ptr if d_irp else None,
            d_ici.ptr if d_ici else None, d_src.ptr, len(sources0), dist_buf.ptr, None))
        return dist_buf.to_host()
    finally:
        for d in (d_rp, d_ci, d_irp, d_ici, d_src):
            if d is not None:
                d.free()


@pytest.mark.parametrize("directed", [False, True])
def test_noalloc_matches_gdistances_twice(directed):
    g = G.rmat(14, 16, seed=5, directed=directed)
    rng = np.random.default_rng(11)
    dist_buf = DeviceArray(np.zeros(g.nv(), np.int32))
    try:
        for sources in (rng.choice(g.nv(), 1).astype(np.int32),
                        rng.choice(g.nv(), 9).astype(np.int32)):
            got = _noalloc_levels(g, sources, dist_buf)
            exp = _device_levels(g, sources)  # handle-based lgbc_gdistances
            assert np.array_equal(got, exp)
    finally:
        dist_buf.free()


def test_noalloc_rejects_oversize_and_bad_sources():
    lib = _lib.lib()
    rc = lib.lgbc_gdistances_noalloc(lgbc_max() + 1, 0, ctypes.c_void_p(1), None, None, None,
                                     None, 0, ctypes.c_void_p(1), None)
    assert rc == _lib.LGBC_EINVAL and "LGBC_NOALLOC_MAX_VERTICES" in _lib.last_error()
    g = lgbc.SimpleGraph.from_edges(4, [(1, 2), (2, 3)])
    dist_buf = DeviceArray(np.zeros(4, np.int32))
    try:
        with pytest.raises(lgbc.ArgumentError):
            _noalloc_levels(g, np.array([7], np.int32), dist_buf)
        # a good call right after a rejected one still matches
        assert np.array_equal(_noalloc_levels(g, np.array([0], np.int32), dist_buf),
                              _device_levels(g, np.array([0], np.int32)))
    finally:
        dist_buf.free()


def lgbc_max():
    return 1 << 22
