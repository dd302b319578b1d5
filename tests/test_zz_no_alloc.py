"""The column filter entry point that allocates nothing (qg_filter_cols_noalloc).

It serves callers that cannot call cudaMalloc -- code inside an allocator or
memory-pool callback, or under a framework that owns all device memory -- so
it takes no qg_ctx and keeps its scratch in a fixed device array inside the
library.  The test calls it through the C ABI and checks its output against the
context-based entry point (qg_filter_cols), bit-exact, on two calls in a row so
that the second call sees the array as the first one left it.  The file is
named to be collected last; it passes alone in a fresh process and after the
other tests.
"""
from ctypes import byref, c_int64, c_void_p

import pytest
import torch

from query_on_opencl_fpga_gb300 import _lib, datagen

pytestmark = pytest.mark.gpu


def _p(t):
    return c_void_p(t.data_ptr())


@pytest.mark.parametrize("n", [100003, 1 << 22])
def test_noalloc_filter_matches_context_filter_twice(n):
    assert torch.cuda.is_available(), "needs a GPU"
    lib = _lib.load()
    stream = torch.cuda.current_stream()
    ctx = c_void_p()
    assert lib.qg_ctx_create(byref(ctx), c_void_p(stream.cuda_stream)) == 0
    try:
        for call, seed in enumerate((n, n + 1)):
            d = datagen.config0_filter(n, seed=seed, device="cuda")
            key, pay, lo, hi = d["key"], d["payload"], d["lo"], d["hi"]
            # existing entry point (allocates through its context)
            ref_out = torch.empty((n, 2), dtype=torch.int32, device="cuda")
            ref_n = c_int64()
            assert lib.qg_filter_cols(ctx, _p(key), _p(pay), n, lo, hi, _p(ref_out), n, byref(ref_n)) == 0
            # the entry point that allocates nothing
            out = torch.full((n, 2), -7, dtype=torch.int32, device="cuda")
            d_n = torch.full((1,), -99, dtype=torch.int64, device="cuda")
            st = lib.qg_filter_cols_noalloc(_p(key), _p(pay), n, lo, hi, _p(out), n, _p(d_n),
                                            c_void_p(stream.cuda_stream))
            assert st == 0, f"call {call}: status {st}"
            torch.cuda.synchronize()
            m = int(d_n.item())
            assert m == ref_n.value, f"call {call}: count {m} != {ref_n.value}"
            assert torch.equal(out[:m], ref_out[:m]), f"call {call}: rows differ"
    finally:
        lib.qg_ctx_destroy(ctx)


def test_noalloc_rejects_oversize():
    lib = _lib.load()
    dummy = torch.zeros(4, dtype=torch.int32, device="cuda")
    d_n = torch.zeros(1, dtype=torch.int64, device="cuda")
    st = lib.qg_filter_cols_noalloc(_p(dummy), _p(dummy), (1 << 26) + 1, 0, 1, _p(dummy), 4, _p(d_n),
                                    c_void_p(0))
    assert st == _lib.QG_ERR_UNSUPPORTED
