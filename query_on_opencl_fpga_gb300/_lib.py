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
    "qg_ctx_timing_span": (ctypes.c_double, [c_void_p]),
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
    "qg_noalloc_set_spin_limit": (c_int, [c_uint32]),
    "qg_noalloc_forget": (c_int, []),
    "qg_scan_excl_i32": (c_int, [c_void_p, c_void_p, c_void_p, c_int64]),
    "qg_sort_rec_by_y": (c_int, [c_void_p, c_void_p, c_int64]),
    "qg_groupby_rec": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_int64,
                               POINTER(c_int64)]),
    "qg_aggregate_groups": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int, c_void_p]),
    "qg_aggregate_group_range": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int64, c_int64,
                                         c_int, c_void_p]),
    "qg_gather_rec": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int64, c_void_p]),
    "qg_scatter_rec": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_int64]),
    "qg_groupby_cols": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_int64,
                                c_void_p, c_void_p, c_void_p, c_int64, c_int, POINTER(c_int64)]),
    "qg_groupby_cols_async": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_int32,
                                      c_int64, c_void_p, c_void_p, c_void_p, c_int64, c_int, c_void_p]),
    "qg_groupby_set_knobs": (c_int, [c_int, c_int, c_int, c_uint32]),
    "qg_groupby_set_single_launch": (c_int, [c_int]),
    "qg_groupby_stats": (c_int, [c_void_p, c_void_p]),
    "qg_join_filter_sort": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_int64,
                                    c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_int64,
                                    POINTER(c_int64)]),
    "qg_steer_attach": (c_int, [c_void_p, c_void_p, ctypes.c_float]),
    "qg_steer_detach": (c_int, [c_void_p]),
    "qg_steer_choose": (c_int, [c_void_p, c_int, c_int64, c_int64, ctypes.c_float, POINTER(c_int),
                                POINTER(ctypes.c_float)]),
    "qg_steer_stats": (c_int, [c_void_p, c_int, c_void_p]),
    "qg_steer_plan": (c_int, [c_void_p, c_int, ctypes.c_float, c_void_p, POINTER(c_int)]),
    "qg_hash_table_bytes": (c_int64, [c_int64]),
    "qg_hash_build_ref": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int64]),
    "qg_hash_probe_ref": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_int64, POINTER(c_int64)]),
    "qg_hash_join_ref": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_int64,
                                 POINTER(c_int64)]),
    "qg_join_set_knobs": (c_int, [c_int, c_int, c_uint32, c_uint32]),
    "qg_join_set_dense": (c_int, [c_int]),
    "qg_sort_set_rank": (c_int, [c_int]),
    "qg_join_stats": (c_int, [c_void_p, c_void_p]),
    "qg_part_model_bytes": (c_int64, []),
    "qg_reduce_rec": (c_int, [c_void_p, c_void_p, c_int64, c_int, POINTER(c_uint32)]),
    "qg_split_rec": (c_int, [c_void_p, c_void_p, c_int64, c_int32, c_void_p, c_void_p]),
    "qg_mlp_param_count": (c_int64, []),
    "qg_mlp_init": (c_int, [c_void_p, c_void_p, c_uint32]),
    "qg_mlp_predict": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p]),
    "qg_mlp_grad": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "qg_mlp_train": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_int, ctypes.c_float,
                             c_void_p, POINTER(c_int), c_void_p]),
    "qg_part_learn": (c_int, [c_void_p, c_void_p, c_int64, c_uint32, c_void_p]),
    "qg_part_eval": (c_int, [c_void_p, c_void_p, c_uint32, c_int, c_void_p, c_int64, c_void_p]),
}

class QgBuf(ctypes.Structure):
    """qg_buf (include/qg_ref.h): the cl_mem stand-in, device pointer + bytes."""
    _fields_ = [("ptr", c_void_p), ("bytes", c_size_t)]


class ScanPara(ctypes.Structure):
    _fields_ = [("pass_", c_uint32), ("gLength", c_uint32), ("blockSize", c_uint32)]


_PB = POINTER(QgBuf)
_PI = POINTER(c_int)
_c = c_int
# The reference's operator surface (include/qg_ref.h).
SIGNATURES.update({
    "qg_ref_last_status": (c_int, []),
    "qg_ref_default_ctx": (c_void_p, []),
    "qg_buf_alloc": (c_int, [_PB, c_size_t]),
    "qg_buf_free": (None, [_PB]),
    "filterImpl": (None, [QgBuf, _c, _c, _PB, _PI, _c, _c, _c, _c, c_void_p]),
    "range_selection": (c_int, [QgBuf, _c, _c, _c, _PB, _c, _c, c_void_p]),
    "CL_RangeSelection": (c_int, [c_void_p, _c, _c, _c, POINTER(c_void_p), _c, _c, _c]),
    "initScan": (None, [_c, POINTER(ScanPara)]),
    "scanImpl": (None, [QgBuf, _c, QgBuf, POINTER(ScanPara), c_void_p]),
    "closeScan": (None, [POINTER(ScanPara)]),
    "radixSortImpl_sm": (None, [QgBuf, _c, _c, _c, _c, c_void_p]),
    "CL_RadixSort": (None, [c_void_p, _c, c_void_p, _c, _c, _c]),
    "groupByImpl": (c_int, [QgBuf, _c, QgBuf, _PB, _c, _c, c_void_p]),
    "CL_GroupBy": (c_int, [c_void_p, _c, c_void_p, POINTER(c_void_p), _c, _c, _c]),
    "parallelAggregate_init": (None, [QgBuf, QgBuf, QgBuf, _c, _c, _c, _c, _c, _c, _c, c_void_p]),
    "aggAfterGroupByImpl": (None, [QgBuf, _c, QgBuf, _c, QgBuf, QgBuf, _c, _c, c_void_p]),
    "CL_agg_max_afterGroupBy": (None, [c_void_p, _c, c_void_p, _c, c_void_p, c_void_p, _c, _c]),
    "CL_agg_min_afterGroupBy": (None, [c_void_p, _c, c_void_p, _c, c_void_p, c_void_p, _c, _c]),
    "CL_agg_sum_afterGroupBy": (None, [c_void_p, _c, c_void_p, _c, c_void_p, c_void_p, _c, _c]),
    "CL_agg_avg_afterGroupBy": (None, [c_void_p, _c, c_void_p, _c, c_void_p, c_void_p, _c, _c]),
    "gatherImpl": (None, [QgBuf, _c, QgBuf, QgBuf, _c, _c, _c, c_void_p]),
    "scatterImpl": (None, [QgBuf, _c, QgBuf, QgBuf, _c, _c, c_void_p]),
    "splitImpl": (None, [QgBuf, _c, _c, QgBuf, QgBuf, _c, _c, _c, c_void_p]),
})

class Query(ctypes.Structure):
    """qg_query (include/qg.h)."""
    _fields_ = [("op", c_int), ("variant", c_int), ("n", c_int64), ("n2", c_int64),
                ("inp", c_void_p * 4), ("lo", c_int32), ("hi", c_int32), ("out", c_void_p * 3),
                ("cap", c_int64), ("d_count", c_void_p)]


SIGNATURES.update({
    "qg_batch_create": (c_int, [POINTER(Query), c_int, c_int, POINTER(c_void_p)]),
    "qg_batch_run": (c_int, [c_void_p, c_void_p]),
    "qg_batch_check": (c_int, [c_void_p, c_void_p]),
    "qg_batch_info": (c_int, [c_void_p, c_void_p]),
    "qg_batch_destroy": (c_int, [c_void_p]),
    "qg_batch_set_lanes": (c_int, [c_int]),
    "qg_batch_set_persistent": (c_int, [c_int]),
})

PLAN_MAX_OPS = 16
PLAN_MAX_IMAGES = 16


class PlanKernel(ctypes.Structure):
    _fields_ = [("kernel_id", c_int), ("variant", c_int)]


class PlanImage(ctypes.Structure):
    _fields_ = [("num_kernels", c_int), ("kernels", PlanKernel * PLAN_MAX_OPS),
                ("luts", c_int), ("regs", c_int), ("rams", c_int), ("dsps", c_int),
                ("total_unit_cost", ctypes.c_float), ("exec_time", ctypes.c_float),
                ("freq", ctypes.c_float), ("mem_inc", ctypes.c_float), ("reconfig_time", ctypes.c_float)]


class Plan(ctypes.Structure):
    _fields_ = [("exec_time", ctypes.c_float), ("image_num", c_int), ("images", PlanImage * PLAN_MAX_IMAGES)]


class PlanVariant(ctypes.Structure):
    _fields_ = [("name", c_char_p), ("kernel_id", c_int), ("lut", c_int), ("reg", c_int), ("ram", c_int),
                ("dsp", c_int), ("unit_cost", ctypes.c_float), ("mem_add", ctypes.c_float),
                ("mem_sub", ctypes.c_float)]


# The planner (include/qg_plan.h); host-only, needs no GPU.
SIGNATURES.update({
    "qg_plan_dp": (c_int, [POINTER(c_int), c_int, ctypes.c_float, POINTER(Plan)]),
    "qg_plan_pipeline": (c_int, [c_int, ctypes.c_float, POINTER(Plan)]),
    "qg_plan_variant_name": (c_char_p, [c_int, c_int]),
    "qg_plan_set_table": (c_int, [POINTER(PlanVariant), c_int, c_int]),
})

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
