"""ctypes binding of libqg.so (the C ABI declared in include/qg.h).

The library is the only compute path: if it is missing or fails to load, this
module raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_int, c_int32, c_int64, c_size_t, c_uint32, c_uint64, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libqg.so"

QG_OK = 0
QG_ERR_INVALID = 1
QG_ERR_CUDA = 2
QG_ERR_CAPACITY = 3
QG_ERR_TABLE_FULL = 4
QG_ERR_TIMEOUT = 5
QG_ERR_OOM = 6
QG_ERR_UNSUPPORTED = 7

QG_REDUCE_SUM, QG_REDUCE_MAX, QG_REDUCE_MIN, QG_REDUCE_AVERAGE = 0, 1, 2, 3
QG_ORDER_NONE, QG_ORDER_KEY = 0, 1

# name -> (restype, argtypes); every symbol include/qg.h declares.
SIGNATURES: dict[str, tuple] = {
    "qg_ctx_create": (c_int, [POINTER(c_void_p), c_void_p]),
    "qg_ctx_destroy": (c_int, [c_void_p]),
    "qg_ctx_set_stream": (c_int, [c_void_p, c_void_p]),
    "qg_ctx_sync": (c_int, [c_void_p]),
    "qg_ctx_set_spin_limit": (c_int, [c_void_p, c_uint32]),
    "qg_ctx_check": (c_int, [c_void_p]),
    "qg_status_string": (c_char_p, [c_int]),
    "qg_last_error_message": (c_char_p, [c_void_p]),
    "qg_ctx_scratch_bytes": (c_size_t, [c_void_p]),
    "qg_ctx_reserve": (c_int, [c_void_p, c_size_t]),
    "qg_ctx_launch_count": (c_uint64, [c_void_p]),
    "qg_ctx_enable_timing": (c_int, [c_void_p, c_int]),
    "qg_ctx_timing_report": (c_int, [c_void_p, c_char_p, c_size_t]),
    "qg_malloc": (c_int, [c_void_p, POINTER(c_void_p), c_size_t]),
    "qg_free": (c_int, [c_void_p, c_void_p]),
    "qg_filter_range_rec": (c_int, [c_void_p, c_void_p, c_int64, c_int32, c_int32, c_void_p, c_int64,
                                    POINTER(c_int64)]),
    "qg_filter_range_rec_async": (c_int, [c_void_p, c_void_p, c_int64, c_int32, c_int32, c_void_p,
                                          c_int64, c_void_p]),
    "qg_filter_cols": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int32, c_int32, c_void_p,
                               c_int64, POINTER(c_int64)]),
    "qg_filter_cols_async": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int32, c_int32,
                                     c_void_p, c_int64, c_void_p]),
    "qg_filter_set_variant": (c_int, [c_int]),
    "qg_filter_cols_noalloc": (c_int, [c_void_p, c_void_p, c_int64, c_int32, c_int32, c_void_p, c_int64,
                                       c_void_p, c_void_p]),
    "qg_scan_excl_i32": (c_int, [c_void_p, c_void_p, c_void_p, c_int64]),
    "qg_sort_rec_by_y": (c_int, [c_void_p, c_void_p, c_int64]),
    "qg_groupby_rec": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_int64,
                               POINTER(c_int64)]),
    "qg_aggregate_groups": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int, c_void_p]),
    "qg_groupby_cols": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_int64,
                                c_void_p, c_void_p, c_void_p, c_int64, c_int, POINTER(c_int64)]),
    "qg_groupby_cols_async": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_int32,
                                      c_int64, c_void_p, c_void_p, c_void_p, c_int64, c_int, c_void_p]),
    "qg_groupby_set_knobs": (c_int, [c_int, c_int, c_int, c_uint32]),
    "qg_groupby_stats": (c_int, [c_void_p, c_void_p]),
    "qg_join_filter_sort": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_int64,
                                    c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_int64,
                                    POINTER(c_int64)]),
    "qg_hash_join_ref": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_int64,
                                 POINTER(c_int64)]),
}

_lib = None


def load() -> ctypes.CDLL:
    """Load libqg.so once and declare every prototype.  Raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -m query_on_opencl_fpga_gb300.build` "
            "(there is no non-CUDA path)")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class QGError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        lib = load()
        name = lib.qg_status_string(status).decode()
        super().__init__(f"{where}: {name} ({status}){': ' + detail if detail else ''}")
