"""The column filter entry point that allocates nothing (qg_filter_cols_noalloc).

It serves callers that cannot call cudaMalloc -- code inside an allocator or
memory-pool callback, or under a framework that owns all device memory -- so
it takes no qg_ctx and keeps its scratch in a fixed device array inside the
library.  The test calls it through the C ABI and checks its output against the
context-based entry point (qg_filter_cols), bit-exact, on two calls in a row so
that the second call sees the array as the first one left it; the other tests
check it against the CPU oracle, its report of a look-back wait that gave up,
a count above the capacity, and calls after its remembered addresses are
dropped.  The file is named to be collected last; it passes alone in a fresh
process and after the other tests.
"""
from ctypes import byref, c_int64, c_void_p

import pytest
import torch

from oracle import oracle as orc
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


def _noalloc(lib, d, n, cap):
    out = torch.full((max(cap, 1), 2), -7, dtype=torch.int32, device="cuda")
    d_n = torch.full((1,), -99, dtype=torch.int64, device="cuda")
    st = lib.qg_filter_cols_noalloc(_p(d["key"]), _p(d["payload"]), n, d["lo"], d["hi"], _p(out), cap, _p(d_n),
                                    c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st, int(d_n.item()), out


@pytest.mark.parametrize("n", [1, 4095, 4097, 300001])
def test_noalloc_filter_matches_oracle(n):
    lib = _lib.load()
    d = datagen.config0_filter(n, seed=7 * n)
    exp = orc.filter_cols(d["key"].numpy(), d["payload"].numpy(), d["lo"], d["hi"])
    dd = {k: (v.cuda() if isinstance(v, torch.Tensor) else v) for k, v in d.items()}
    st, m, out = _noalloc(lib, dd, n, n)
    assert st == 0 and m == exp.shape[0]
    assert (out[:m].cpu().numpy() == exp).all()


def test_noalloc_count_above_capacity_is_reported_not_an_error():
    # QG_OK with only `cap` pairs written; *d_out_n is the full count
    lib = _lib.load()
    n = 1 << 18
    d = datagen.config0_filter(n, seed=3, device="cuda")
    exp = orc.filter_cols(d["key"].cpu().numpy(), d["payload"].cpu().numpy(), d["lo"], d["hi"])
    cap = exp.shape[0] // 2
    st, m, out = _noalloc(lib, d, n, cap)
    assert st == 0 and m == exp.shape[0]
    assert (out[:cap].cpu().numpy() == exp[:cap]).all()


def test_noalloc_timeout_is_reported_and_next_call_exact():
    # A poll limit of 0 makes every waiting tile give up at once: the call
    # reports -QG_ERR_TIMEOUT through the count; with the default limit the
    # next call is exact again (the error word was cleared by the report).
    lib = _lib.load()
    n = 1 << 20
    d = datagen.config0_filter(n, seed=11, device="cuda")
    exp = orc.filter_cols(d["key"].cpu().numpy(), d["payload"].cpu().numpy(), d["lo"], d["hi"])
    assert lib.qg_noalloc_set_spin_limit(0) == 0
    try:
        st, m, _ = _noalloc(lib, d, n, n)
        assert st == 0 and m == -_lib.QG_ERR_TIMEOUT
    finally:
        lib.qg_noalloc_set_spin_limit(1 << 22)
    st, m, out = _noalloc(lib, d, n, n)
    assert st == 0 and m == exp.shape[0]
    assert (out[:m].cpu().numpy() == exp).all()


def test_noalloc_after_forget_looks_the_address_up_again():
    lib = _lib.load()
    n = 1 << 16
    d = datagen.config0_filter(n, seed=13, device="cuda")
    exp = orc.filter_cols(d["key"].cpu().numpy(), d["payload"].cpu().numpy(), d["lo"], d["hi"])
    assert lib.qg_noalloc_forget() == 0
    st, m, out = _noalloc(lib, d, n, n)
    assert st == 0 and m == exp.shape[0]
    assert (out[:m].cpu().numpy() == exp).all()
