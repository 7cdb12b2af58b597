"""ctypes binding of ``liblgbc.so`` (the C ABI declared in include/lgbc.h).

The library is built in-tree by ``lightgraphs.jl_gb300/build.py``.  Loading
fails loudly when it is missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os
import threading

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG, "lib", "liblgbc.so")

LGBC_OK = 0
LGBC_EINVAL = -1
LGBC_ENOMEM = -2
LGBC_ECUDA = -3
LGBC_ETIMEOUT = -4
UNREACHED = 2**31 - 1

_lock = threading.Lock()
_lib = None


class LGBCError(RuntimeError):
    """A CUDA-side failure (no device, launch failure, out of memory, timeout)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"lgbc error {code}: {msg}")
        self.code = code


class ArgumentError(ValueError):
    """Julia's ArgumentError (e.g. ``sample`` with k > n, src/utils.jl:14)."""


class BoundsError(IndexError):
    """Julia's BoundsError (a vertex id outside 1:nv(g))."""


class MethodError(TypeError):
    """Julia's MethodError: an argument combination the GPU path does not cover
    (a distance matrix other than DefaultDistance)."""


class LgbcStats(ctypes.Structure):
    _fields_ = [("kernel_launches", ctypes.c_int64), ("batches", ctypes.c_int64),
                ("levels", ctypes.c_int64), ("active_sources", ctypes.c_int64),
                ("wide_batches", ctypes.c_int64), ("topdown_levels", ctypes.c_int64),
                ("bottomup_levels", ctypes.c_int64)]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_}


class LgbcTuning(ctypes.Structure):
    _fields_ = [("alpha", ctypes.c_double), ("beta", ctypes.c_double),
                ("hub_degree", ctypes.c_int32), ("lanes", ctypes.c_int32),
                ("dense_edges", ctypes.c_int32), ("segment_degree", ctypes.c_int32),
                ("source_order", ctypes.c_int32), ("graph_loop", ctypes.c_int32),
                ("stack_vertices", ctypes.c_int32), ("hub_order", ctypes.c_int32),
                ("dependency_df32", ctypes.c_int32)]


class LgbcTrainCfg(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int32), ("batch", ctypes.c_int32), ("warmup", ctypes.c_int32),
                ("lr", ctypes.c_float), ("lr_final", ctypes.c_float), ("beta1", ctypes.c_float),
                ("beta2", ctypes.c_float), ("eps", ctypes.c_float), ("seed", ctypes.c_uint64)]


SAMPLE_IID = 0
SAMPLE_SYSTEMATIC = 1
MLP_PARAMS = 4545
MLP_HIDDEN = 64
MLP_FEATURES = 4


def _declare(lib) -> None:
    c_int, i64, p = ctypes.c_int, ctypes.c_int64, ctypes.c_void_p
    pp = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "lgbc_version": ([], ctypes.c_char_p),
        "lgbc_last_error": ([], ctypes.c_char_p),
        "lgbc_device_count": ([], c_int),
        "lgbc_graph_create": ([pp, i64, i64, p, p, p, p, c_int], c_int),
        "lgbc_graph_destroy": ([p], c_int),
        "lgbc_graph_info": ([p, ctypes.POINTER(i64), ctypes.POINTER(i64),
                             ctypes.POINTER(c_int)], c_int),
        "lgbc_gdistances": ([p, p, i64, p], c_int),
        "lgbc_gdistances_batch": ([p, p, i64, p], c_int),
        "lgbc_betweenness": ([p, p, i64, c_int, p], c_int),
        "lgbc_path_counts": ([p, p, i64, p, p], c_int),
        "lgbc_betweenness_dev": ([p, p, i64, c_int, p], c_int),
        "lgbc_graph_sync": ([p], c_int),
        "lgbc_timer_start": ([p], c_int),
        "lgbc_timer_stop": ([p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(i64)], c_int),
        "lgbc_graph_stats": ([p, ctypes.POINTER(LgbcStats)], c_int),
        "lgbc_get_tuning": ([p, ctypes.POINTER(LgbcTuning)], c_int),
        "lgbc_set_tuning": ([p, ctypes.POINTER(LgbcTuning)], c_int),
        "lgbc_tune": ([p, ctypes.c_char_p], c_int),
        "lgbc_device_alloc": ([pp, i64], c_int),
        "lgbc_device_free": ([p], c_int),
        "lgbc_host_alloc": ([pp, i64], c_int),
        "lgbc_host_free": ([p], c_int),
        "lgbc_memcpy": ([p, p, i64, c_int], c_int),
        "lgbc_gdistances_noalloc": ([i64, i64, p, p, p, p, p, i64, p, p], c_int),
        "lgbc_graph_create_from_edges": ([pp, i64, i64, p, p, c_int], c_int),
        "lgbc_graph_csr": ([p, p, p, p, p], c_int),
        "lgbc_betweenness_many": ([i64, p, p, p, p, p, c_int, p], c_int),
        "lgbc_core_number": ([p, p], c_int),
        "lgbc_features": ([p, p], c_int),
        "lgbc_dependency_mass": ([p, p, i64, p], c_int),
        "lgbc_distance_stats": ([p, p, i64, p, p, p], c_int),
        "lgbc_stress": ([p, p, i64, p], c_int),
        "lgbc_bfs_parents": ([p, ctypes.c_int32, c_int, p], c_int),
        "lgbc_has_path": ([p, ctypes.c_int32, ctypes.c_int32, p, i64, ctypes.POINTER(c_int)], c_int),
        "lgbc_betweenness_weighted": ([p, p, p, i64, p], c_int),
        "lgbc_mlp_create": ([pp, ctypes.c_uint64], c_int),
        "lgbc_mlp_destroy": ([p], c_int),
        "lgbc_mlp_get_params": ([p, p, p], c_int),
        "lgbc_mlp_set_params": ([p, p], c_int),
        "lgbc_mlp_set_norm": ([p, p, p], c_int),
        "lgbc_mlp_get_norm": ([p, p, p], c_int),
        "lgbc_mlp_forward": ([p, p, i64, p], c_int),
        "lgbc_mlp_grad": ([p, p, p, i64, p, p], c_int),
        "lgbc_mlp_train": ([p, p, p, i64, p, i64, ctypes.POINTER(LgbcTrainCfg), p], c_int),
        "lgbc_proposal_build": ([p, p, ctypes.c_double, p], c_int),
        "lgbc_proposal_sample": ([p, i64, ctypes.c_uint64, c_int, p, p], c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res


def lib():
    """Load (once) and return the CUDA library; raise if it was never built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise LGBCError(LGBC_ECUDA,
                                f"{LIB_PATH} is missing: build it with "
                                "`python lightgraphs.jl_gb300/build.py` (there is no CPU fallback)")
            h = ctypes.CDLL(LIB_PATH)
            _declare(h)
            _lib = h
        return _lib


def last_error() -> str:
    return lib().lgbc_last_error().decode(errors="replace")


def check(rc: int) -> None:
    """Map a C return code onto the Julia-style exception hierarchy."""
    if rc == LGBC_OK:
        return
    msg = last_error()
    if rc == LGBC_EINVAL:
        raise ArgumentError(msg)
    raise LGBCError(rc, msg)


def ptr(a) -> ctypes.c_void_p | None:
    """Address of a contiguous numpy array (None for None)."""
    if a is None:
        return None
    return ctypes.c_void_p(a.ctypes.data)
