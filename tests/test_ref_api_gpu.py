"""The reference operator surface (include/qg_ref.h) driven the way the
reference's own test drivers drive it (host/host/test*.cpp), checked against
the golden vectors made from the reference's generator and validators."""
import ctypes
import hashlib
from ctypes import byref, c_int, c_void_p

import numpy as np
import pytest
import torch

from query_on_opencl_fpga_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    L = _lib.load()
    assert L.qg_ref_default_ctx()
    return L


def host_ptr(a):
    return c_void_p(a.ctypes.data)


def dbuf(t):
    return _lib.QgBuf(t.data_ptr(), t.numel() * t.element_size())


def take_host_array(ptr, n, dtype):
    """Copy then free a malloc'ed host array returned by a CL_* wrapper."""
    if n == 0:
        return np.zeros((0,), dtype)
    buf = (ctypes.c_char * (n * np.dtype(dtype).itemsize)).from_address(ptr.value)
    out = np.frombuffer(bytes(buf), dtype).copy()
    ctypes.CDLL(None).free(ptr)
    return out


def test_testFilterImpl_flow(lib, orc, golden):
    # testFilter.cpp:197-232: generateRand(Rin, 100, rLen, 0); smallKey = rand()%100;
    # largeKey = min(smallKey+6, 100); CL_RangeSelection; validateFilter.
    meta, arrs = golden
    c = meta["cases"]["filter"]
    rin = orc.generate_rand(100, c["n"], 0)
    hout = c_void_p()
    out_n = lib.CL_RangeSelection(host_ptr(rin), c["n"], c["small"], c["large"], byref(hout), 256, 128, 0)
    assert out_n == c["out_n"], lib.qg_ref_last_status()
    got = take_host_array(hout, out_n * 2, np.int32).reshape(-1, 2)
    assert np.array_equal(got, arrs["filter_out"])


def _from_device(ptr, nrec):
    """Copy `nrec` records at a raw device pointer into a tensor (identity gather)."""
    L = _lib.load()
    t = torch.empty((nrec, 2), dtype=torch.int32, device="cuda")
    loc = torch.arange(nrec, dtype=torch.int32, device="cuda")
    assert L.qg_gather_rec(L.qg_ref_default_ctx(), c_void_p(ptr), nrec, c_void_p(loc.data_ptr()), 1, nrec,
                           c_void_p(t.data_ptr())) == 0
    torch.cuda.synchronize()
    return t


def test_filterImpl_device_and_beginpos(lib, orc):
    # filterImpl allocates *d_Rout (rLen records) and filters d_Rin[beginPos, beginPos + rLen)
    rin = orc.generate_rand(1000, 50000, 5)
    d = torch.from_numpy(rin).cuda()
    out = _lib.QgBuf()
    n = c_int()
    lib.filterImpl(dbuf(d), 1000, 40000, byref(out), byref(n), 256, 128, 100, 300, None)
    assert lib.qg_ref_last_status() == 0
    assert out.bytes == 40000 * 8
    exp = orc.filter_rec(rin[1000:41000], 100, 300)
    assert n.value == exp.shape[0]
    got = _from_device(out.ptr, n.value).cpu().numpy()
    assert np.array_equal(got, exp)
    lib.qg_buf_free(byref(out))
    # range_selection returns the count
    out2 = _lib.QgBuf()
    assert lib.range_selection(dbuf(d), 50000, 100, 300, byref(out2), 256, 128, None) == \
        orc.filter_rec(rin, 100, 300).shape[0]
    lib.qg_buf_free(byref(out2))


def test_testScanImpl_flow(lib, orc, golden):
    # testScan.cpp:342-390: generateRandInt(Rin, rLen, rLen, 0); initScan; scanImpl; validateScan
    meta, _ = golden
    s = meta["cases"]["scan"]
    sin = orc.generate_rand_int(s["n"], s["n"], 0)
    d_in = torch.from_numpy(sin).cuda()
    d_out = torch.empty_like(d_in)
    sp = _lib.ScanPara()
    lib.initScan(s["n"], byref(sp))
    assert sp.blockSize == 256 and sp.gLength == s["n"]
    lib.scanImpl(dbuf(d_in), s["n"], dbuf(d_out), byref(sp), None)
    lib.closeScan(byref(sp))
    assert lib.qg_ref_last_status() == 0
    assert hashlib.sha256(d_out.cpu().numpy().tobytes()).hexdigest() == s["output_sha"]


@pytest.mark.parametrize("n", [2048, 1 << 15, 100003])
def test_testSortImpl_flow(lib, orc, golden, n):
    # testSort.cpp:276-296: generateRand(Rin, 200, rLen, 0); CL_RadixSort; validateSort
    meta, _ = golden
    c = meta["cases"][f"sort_{n}"]
    rin = orc.generate_rand(200, n, 0)
    hout = np.empty_like(rin)
    lib.CL_RadixSort(host_ptr(rin), n, host_ptr(hout), 256, 128, 0)
    assert lib.qg_ref_last_status() == 0
    assert hashlib.sha256(np.ascontiguousarray(hout[:, 1]).tobytes()).hexdigest() == c["keys_sorted_sha"]


def test_testGroupByImpl_flow(lib, orc, golden):
    # testGroupBy.cpp:156-175: generateRand(Rin, 64, rLen, 0); CL_GroupBy; validateGroupBy
    meta, arrs = golden
    c = meta["cases"]["groupby"]
    rin = orc.generate_rand(64, c["n"], 0)
    rin[:, 1] = np.mod(rin[:, 1], 64)
    hout = np.empty_like(rin)
    hsp = c_void_p()
    g = lib.CL_GroupBy(host_ptr(rin), c["n"], host_ptr(hout), byref(hsp), 256, 128, 0)
    assert g == c["num_groups"]
    sp = take_host_array(hsp, g, np.int32)
    assert np.array_equal(sp, arrs["groupby_startpos"])
    assert np.array_equal(hout[:, 1], orc.sort_rec(rin)[:, 1])


@pytest.mark.parametrize("op,name", [(0, "sum"), (1, "max"), (2, "min"), (3, "avg")])
def test_testAggAfterGroupByImpl_flow(lib, orc, golden, op, name):
    # testAggAfterGB.cpp:127-255: groupByImpl(d_Rout, rLen, d_Rout, &d_startPos, ...) then
    # parallelAggregate_init over chunks of MAX_NUM_BLOCK = 512 groups.
    meta, arrs = golden
    c = meta["cases"]["aggregate"]
    rin = orc.generate_rand(50, c["n"], 0)
    rin[:, 1] = np.mod(rin[:, 1], 50)
    d = torch.from_numpy(rin).cuda()
    sp = _lib.QgBuf()
    g = lib.groupByImpl(dbuf(d), c["n"], dbuf(d), byref(sp), 256, 128, None)
    assert g == c["num_groups"]
    agg = torch.empty(g, dtype=torch.int32, device="cuda")
    for chunk in range((g + 511) // 512):
        nb = min(512, g - chunk * 512)
        lib.parallelAggregate_init(dbuf(d), sp, dbuf(agg), op, chunk * 512, g, nb, 256, 1024, c["n"], None)
        assert lib.qg_ref_last_status() == 0
    assert np.array_equal(agg.cpu().numpy(), arrs[f"agg_{name}"])
    lib.qg_buf_free(byref(sp))


@pytest.mark.parametrize("fn,op,name", [("CL_agg_sum_afterGroupBy", 0, "sum"), ("CL_agg_max_afterGroupBy", 1, "max"),
                                        ("CL_agg_min_afterGroupBy", 2, "min"), ("CL_agg_avg_afterGroupBy", 3, "avg")])
def test_CL_agg_afterGroupBy(lib, orc, golden, fn, op, name):
    # AggAfterGroupBy.cpp:30-170 with Ragg[i] = (i, i): the gathered S[i].x is the
    # sorted record's row id, so the result equals the golden aggregate.
    meta, arrs = golden
    c = meta["cases"]["aggregate"]
    n = c["n"]
    rin = orc.generate_rand(50, n, 0)
    rin[:, 1] = np.mod(rin[:, 1], 50)
    srt = orc.sort_rec(rin)
    sp = orc.group_startpos(srt)
    ragg = np.stack([np.arange(n, dtype=np.int32)] * 2, axis=1)
    out = np.zeros(sp.size, np.int32)
    getattr(lib, fn)(host_ptr(srt), n, host_ptr(sp), sp.size, host_ptr(ragg), host_ptr(out), 256, 0)
    assert lib.qg_ref_last_status() == 0
    assert np.array_equal(out, arrs[f"agg_{name}"])


def test_gather_scatter(lib):
    rng = np.random.default_rng(7)
    n = 100003
    R = rng.integers(-(2 ** 31), 2 ** 31, (n, 2), dtype=np.int64).astype(np.int32)
    loc = rng.permutation(n).astype(np.int32)
    loc[::97] = -5  # out of range: left untouched
    dR, dloc = torch.from_numpy(R).cuda(), torch.from_numpy(loc).cuda()
    S = torch.full((n, 2), 11, dtype=torch.int32, device="cuda")
    lib.gatherImpl(dbuf(dR), n, dbuf(dloc), dbuf(S), n, 256, 128, None)
    exp = np.full((n, 2), 11, np.int32)
    ok = loc >= 0
    exp[ok] = R[loc[ok]]
    assert np.array_equal(S.cpu().numpy(), exp)
    T = torch.full((n, 2), 3, dtype=torch.int32, device="cuda")
    lib.scatterImpl(dbuf(dR), n, dbuf(dloc), dbuf(T), 256, 128, None)
    exp2 = np.full((n, 2), 3, np.int32)
    exp2[loc[ok]] = R[ok]
    assert np.array_equal(T.cpu().numpy(), exp2)


def test_errors_return_status_not_exit(lib):
    n = c_int()
    lib.filterImpl(_lib.QgBuf(None, 0), 0, -5, None, byref(n), 256, 128, 0, 1, None)
    assert lib.qg_ref_last_status() == _lib.QG_ERR_INVALID
