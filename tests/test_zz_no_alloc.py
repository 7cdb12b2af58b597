"""lgbc_gdistances_noalloc: gdistances for callers that cannot allocate.

Some callers cannot call cudaMalloc: a host whose device memory belongs to
another allocator with a fixed budget (a Julia CuArray pool, a serving process
that reserves the GPU's memory when it starts), or a loop that must not pay
cudaFree's device-wide synchronisation.  This entry point takes every input
and output as caller-owned device pointers and keeps its BFS scratch in a
fixed static device array.  The test (only the test, never the entry point)
allocates the device buffers, calls the entry point twice in a row through
the C ABI with different sources, and checks each result bit for bit against
the handle-based lgbc_gdistances and the CPU oracle.  It also checks that a
malformed CSR or source is rejected before any BFS kernel runs, a call on a
non-default stream, and a graph too large for the shared-memory frontier
bitmap.  It lives in its own file, collected last.
"""
import ctypes

import numpy as np
import pytest

import lgbc
from lgbc import _lib
from lgbc import generators as G
from lgbc.traversals import _device_levels
from oracle import oracle

pytestmark = pytest.mark.gpu

MAX_VERTICES = 1 << 22  # LGBC_NOALLOC_MAX_VERTICES


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


def _noalloc_levels(n, rp, ci, sources0, dist_buf, irp=None, ici=None, stream=None):
    lib = _lib.lib()
    d_rp, d_ci = DeviceArray(rp), DeviceArray(ci)
    d_irp = d_ici = None
    if irp is not None:
        d_irp, d_ici = DeviceArray(irp), DeviceArray(ici)
    d_src = DeviceArray(np.asarray(sources0, np.int32))
    try:
        _lib.check(lib.lgbc_gdistances_noalloc(
            n, len(ci), d_rp.ptr, d_ci.ptr, d_irp.ptr if d_irp else None,
            d_ici.ptr if d_ici else None, d_src.ptr, len(sources0), dist_buf.ptr,
            ctypes.c_void_p(stream) if stream else None))
        return dist_buf.to_host()
    finally:
        for d in (d_rp, d_ci, d_irp, d_ici, d_src):
            if d is not None:
                d.free()


def _graph_levels(g, sources0, dist_buf, stream=None):
    rp, ci = g.csr()
    irp = ici = None
    if g.is_directed():
        irp, ici = g.in_csr()
    return _noalloc_levels(g.nv(), rp, ci, sources0, dist_buf, irp, ici, stream)


def _oracle_levels(g, sources0):
    rp, ci = g.csr()
    return oracle.gdistances(rp, ci, sources0)


@pytest.mark.parametrize("directed", [False, True])
def test_noalloc_matches_gdistances_twice(directed):
    g = G.rmat(14, 16, seed=5, directed=directed)
    rng = np.random.default_rng(11)
    dist_buf = DeviceArray(np.zeros(g.nv(), np.int32))
    try:
        for sources in (rng.choice(g.nv(), 1).astype(np.int32),
                        rng.choice(g.nv(), 9).astype(np.int32)):
            got = _graph_levels(g, sources, dist_buf)
            assert np.array_equal(got, _device_levels(g, sources))  # handle-based lgbc_gdistances
            assert np.array_equal(got, _oracle_levels(g, sources))
    finally:
        dist_buf.free()


def test_noalloc_unstaged_bitmap_and_stream():
    # 2^21 vertices: the frontier bitmap (256 KB) exceeds one block's shared
    # memory, so the bottom-up levels read it from global memory; the second
    # call runs on a stream of the caller's (a torch stream here)
    torch = pytest.importorskip("torch")
    g = G.rmat(21, 4, seed=9)
    assert (g.nv() + 31) // 32 * 4 > 227 * 1024 and g.nv() <= MAX_VERTICES
    deg = g.degrees()
    src = np.flatnonzero(deg > 0)[[0, 1000, 50000]].astype(np.int32)
    dist_buf = DeviceArray(np.zeros(g.nv(), np.int32))
    try:
        exp = _oracle_levels(g, src)
        assert np.array_equal(_graph_levels(g, src, dist_buf), exp)
        s = torch.cuda.Stream()
        assert np.array_equal(_graph_levels(g, src, dist_buf, stream=s.cuda_stream), exp)
    finally:
        dist_buf.free()


def test_noalloc_rejects_bad_inputs():
    lib = _lib.lib()
    rc = lib.lgbc_gdistances_noalloc(MAX_VERTICES + 1, 0, ctypes.c_void_p(1), None, None, None,
                                     None, 0, ctypes.c_void_p(1), None)
    assert rc == _lib.LGBC_EINVAL and "LGBC_NOALLOC_MAX_VERTICES" in _lib.last_error()
    g = lgbc.SimpleGraph.from_edges(4, [(1, 2), (2, 3)])
    rp, ci = g.csr()
    dist_buf = DeviceArray(np.zeros(4, np.int32))
    try:
        with pytest.raises(lgbc.ArgumentError):
            _graph_levels(g, np.array([7], np.int32), dist_buf)  # source outside [0, n)
        bad = rp.copy()
        bad[-1] = len(ci) + 1  # rowptr[n] past nnz: rejected before any BFS kernel reads colidx
        with pytest.raises(lgbc.ArgumentError):
            _noalloc_levels(4, bad, ci, np.array([0], np.int32), dist_buf)
        bad = rp.copy()
        bad[0] = -1
        with pytest.raises(lgbc.ArgumentError):
            _noalloc_levels(4, bad, ci, np.array([0], np.int32), dist_buf)
        # a good call right after a rejected one still matches
        src = np.array([0], np.int32)
        got = _graph_levels(g, src, dist_buf)
        assert np.array_equal(got, _device_levels(g, src))
        assert np.array_equal(got, _oracle_levels(g, src))
    finally:
        dist_buf.free()
