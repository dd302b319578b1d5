"""GB300-native relational-operator hot path (filter, scan, sort, group-by +
aggregation, fused filter+aggregation, hash join + filter + sort) behind the
reference operator interface of Xtra-Computing/Query_on_OpenCL_FPGA.

All compute runs in libqg.so (hand-written CUDA for sm_103a, C ABI in
include/qg.h).  Importing the package does not load the library; the first
operator call does, and fails loudly if it is missing.
"""
from ._lib import LIB_PATH, QGError, load  # noqa: F401

__all__ = ["LIB_PATH", "QGError", "load"]
