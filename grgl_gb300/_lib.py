"""ctypes binding of libgrgx.so (include/grgx.h).

The library is built in-tree (grgl_gb300/build.py).  Loading fails loudly when it is missing:
there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libgrgx.so"

OK, ERR_API_MISUSE, ERR_CUDA, ERR_OOM, ERR_BAD_FILE, ERR_UNSUPPORTED, ERR_NO_DEVICE, ERR_TIMEOUT = range(8)
FLAG_DEVICE_POINTERS, FLAG_F32_PLAIN, FLAG_SYNC, FLAG_OVERWRITE, FLAG_F64_NATIVE = 0x1, 0x2, 0x4, 0x8, 0x10
FLAG_NO_GRAPH = 0x20
FLAG_ASYNC = 0x40
REQUEST_STANDARDIZED = 0x1
REQUEST_BY_INDIVIDUAL = 0x2
NOALLOC_SCRATCH_BYTES = 64 << 20  # GRGX_NOALLOC_SCRATCH_BYTES

# Every symbol include/grgx.h declares, with its ctypes signature.
c_graph_p = ctypes.c_void_p
_u64, _u32, _int, _vp = ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, ctypes.c_void_p


class GraphInfo(ctypes.Structure):
    _fields_ = [(name, _u64) for name in ("num_nodes", "num_edges", "num_samples", "num_mutations", "ploidy",
                                          "num_levels", "has_missing", "has_coals", "device_bytes")]


class Timing(ctypes.Structure):
    _fields_ = [("total_ms", ctypes.c_float), ("sweep_ms", ctypes.c_float), ("launches", _u64),
                ("alg_bytes", _u64)]


class Request(ctypes.Structure):
    _fields_ = [("dtype", ctypes.c_int), ("direction", ctypes.c_int), ("rows", _u64), ("input", _vp),
                ("output", _vp), ("options", _u32)]


class RequestStats(ctypes.Structure):
    _fields_ = [("submit_s", ctypes.c_double), ("start_s", ctypes.c_double), ("done_s", ctypes.c_double),
                ("batch_requests", _u64), ("batch_rows", _u64)]


SIGNATURES = {
    "grgx_last_error": (ctypes.c_char_p, []),
    "grgx_version": (ctypes.c_char_p, []),
    "grgx_graph_load": (_int, [ctypes.c_char_p, ctypes.POINTER(c_graph_p)]),
    "grgx_graph_from_csr": (_int, [_u64, _u64, _u64, _vp, _vp, _u64, _vp, _vp, _vp, ctypes.POINTER(c_graph_p)]),
    "grgx_graph_generate": (_int, [_u64, _u64, _u64, _u32, _int, ctypes.POINTER(c_graph_p)]),
    "grgx_graph_save": (_int, [c_graph_p, ctypes.c_char_p]),
    "grgx_graph_destroy": (None, [c_graph_p]),
    "grgx_graph_subset": (_int, [c_graph_p, _vp, _u64, ctypes.POINTER(c_graph_p)]),
    "grgx_graph_info_get": (_int, [c_graph_p, ctypes.POINTER(GraphInfo)]),
    "grgx_graph_export": (_int, [c_graph_p, _vp, _vp, _vp, _vp, _vp]),
    "grgx_graph_upload": (_int, [c_graph_p]),
    "grgx_matmul": (_int, [c_graph_p, _int, _vp, _u64, _u64, _int, _vp, _u64, _int, _int, _vp, _int, _vp, _u32,
                           _vp]),
    "grgx_matmul_noalloc": (_int, [c_graph_p, _int, _vp, _u64, _u64, _int, _vp, _u64, _vp]),
    "grgx_matmul_batch": (_int, [c_graph_p, ctypes.POINTER(Request), _u64, _u64, _u32, _vp]),
    "grgx_matmul_standardized": (_int, [c_graph_p, _int, _vp, _u64, _u64, _int, _vp, _u64, _u32, _vp]),
    "grgx_matmul_gram": (_int, [c_graph_p, _int, _vp, _u64, _u64, _int, _vp, _u64, _int, _u32, _vp]),
    "grgx_server_create": (_int, [_u32, _u64, _u64, ctypes.POINTER(_vp)]),
    "grgx_server_add_graph": (_int, [_vp, c_graph_p, ctypes.POINTER(_u32)]),
    "grgx_server_submit": (_int, [_vp, _u32, ctypes.POINTER(Request), ctypes.POINTER(_u64)]),
    "grgx_server_wait": (_int, [_vp, _u64, ctypes.c_double, ctypes.POINTER(RequestStats)]),
    "grgx_server_destroy": (None, [_vp]),
    "grgx_pool_usage": (_int, [_int, ctypes.POINTER(_u64), ctypes.POINTER(_u64)]),
    "grgx_measure_l2_bandwidth": (_int, [_u64, _int, ctypes.POINTER(ctypes.c_double)]),
    "grgx_host_alloc": (_int, [_u64, ctypes.POINTER(_vp)]),
    "grgx_host_free": (None, [_vp]),
    "grgx_autotune": (_int, [c_graph_p, _int, _u64, _int, _u32, ctypes.c_char_p, _u64, ctypes.POINTER(_u64)]),
    "grgx_autotune_export": (_int, [ctypes.c_char_p, _u64, ctypes.POINTER(_u64)]),
    "grgx_autotune_import": (_int, [ctypes.c_char_p]),
    "grgx_autotune_clear": (None, []),
    "grgx_set_timing": (None, [_int]),
    "grgx_last_timing": (_int, [ctypes.POINTER(Timing)]),
    "grgx_collect_timings": (_int, [ctypes.POINTER(Timing), _u64, ctypes.POINTER(_u64)]),
}

_lib = None
_lock = threading.Lock()


def lib() -> ctypes.CDLL:
    """Load libgrgx.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise ImportError(f"{LIB_PATH} is missing: build it with grgl_gb300.build.build()")
            handle = ctypes.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
    return _lib


def last_error() -> str:
    return lib().grgx_last_error().decode()


def check(status: int):
    """Raise the exception the reference binding raises for this status."""
    if status == OK:
        return
    msg = last_error()
    if status == ERR_OOM:
        raise MemoryError(msg)
    raise RuntimeError(msg)
