"""ctypes binding of the CPU oracle (oracle/liboracle.so, built from
oracle/qg_oracle.c by oracle/build_ref.sh).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / --impl reference legs of bench.py, never by the product.
"""
from __future__ import annotations

import ctypes
import subprocess
from ctypes import c_int, c_int32, c_int64, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_TOOL = HERE / "_ref" / "ref_tool"

_lib = None


def build() -> None:
    subprocess.run(["bash", str(HERE / "build_ref.sh")], check=True)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = ctypes.CDLL(str(LIB))
        sig = {
            "orc_num_threads": (c_int, []),
            "orc_set_threads": (None, [c_int]),
            "orc_generate_rand": (None, [c_void_p, c_int, c_int64, c_int]),
            "orc_generate_rand_int": (None, [c_void_p, c_int, c_int64, c_int]),
            "orc_filter_rec": (c_int64, [c_void_p, c_int64, c_int32, c_int32, c_void_p]),
            "orc_filter_cols": (c_int64, [c_void_p, c_void_p, c_int64, c_int32, c_int32, c_void_p]),
            "orc_filter_cols_mt": (c_int64, [c_void_p, c_void_p, c_int64, c_int32, c_int32, c_void_p]),
            "orc_scan_excl_i32": (None, [c_void_p, c_int64, c_void_p]),
            "orc_sort_rec_by_y": (None, [c_void_p, c_int64]),
            "orc_group_startpos": (c_int64, [c_void_p, c_int64, c_void_p]),
            "orc_aggregate_groups": (None, [c_void_p, c_int64, c_void_p, c_int64, c_int, c_void_p]),
            "orc_groupby_cols": (c_int64, [c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_int64,
                                           c_int64, c_void_p, c_void_p, c_void_p]),
            "orc_groupby_cols_mt": (c_int64, [c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_int64,
                                              c_int64, c_void_p, c_void_p, c_void_p]),
            "orc_join_filter_sort": (c_int64, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_int64,
                                               c_int32, c_int32, c_int64, c_void_p, c_void_p, c_void_p]),
            "orc_join_filter_sort_mt": (c_int64, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p,
                                                  c_int64, c_int32, c_int32, c_int64, c_void_p,
                                                  c_void_p, c_void_p]),
            "orc_hash_join_ref": (c_int64, [c_void_p, c_int64, c_void_p, c_int64, c_int64, c_void_p]),
            "orc_mlp_forward": (None, [c_void_p, c_void_p, c_int64, c_void_p]),
            "orc_reduce_rec": (ctypes.c_uint32, [c_void_p, c_int64, c_int]),
            "orc_split_rec": (None, [c_void_p, c_int64, c_int32, c_void_p, c_void_p]),
            "orc_mlp_grad": (ctypes.c_double, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray | None) -> c_void_p:
    if a is None:
        return c_void_p(0)
    assert a.flags["C_CONTIGUOUS"]
    return c_void_p(a.ctypes.data)


def threads() -> int:
    return lib().orc_num_threads()


def set_threads(t: int) -> None:
    lib().orc_set_threads(t)


def generate_rand(maxmax: int, n: int, seed: int) -> np.ndarray:
    r = np.empty((n, 2), np.int32)
    lib().orc_generate_rand(_p(r), maxmax, n, seed)
    return r


def generate_rand_int(maxv: int, n: int, seed: int) -> np.ndarray:
    r = np.empty(n, np.int32)
    lib().orc_generate_rand_int(_p(r), maxv, n, seed)
    return r


def filter_rec(rec: np.ndarray, lo: int, hi: int) -> np.ndarray:
    rec = np.ascontiguousarray(rec, np.int32)
    out = np.empty_like(rec)
    k = lib().orc_filter_rec(_p(rec), rec.shape[0], lo, hi, _p(out))
    return out[:k]


def filter_cols(key: np.ndarray, pay: np.ndarray, lo: int, hi: int, mt: bool = False) -> np.ndarray:
    key = np.ascontiguousarray(key, np.int32)
    pay = np.ascontiguousarray(pay, np.int32)
    out = np.empty((key.size, 2), np.int32)
    f = lib().orc_filter_cols_mt if mt else lib().orc_filter_cols
    k = f(_p(key), _p(pay), key.size, lo, hi, _p(out))
    return out[:k]


def scan_excl(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.int32)
    out = np.empty_like(x)
    lib().orc_scan_excl_i32(_p(x), x.size, _p(out))
    return out


def sort_rec(rec: np.ndarray) -> np.ndarray:
    r = np.array(rec, np.int32, copy=True, order="C")
    lib().orc_sort_rec_by_y(_p(r), r.shape[0])
    return r


def group_startpos(sorted_rec: np.ndarray) -> np.ndarray:
    sorted_rec = np.ascontiguousarray(sorted_rec, np.int32)
    sp = np.empty(max(sorted_rec.shape[0], 1), np.int32)
    g = lib().orc_group_startpos(_p(sorted_rec), sorted_rec.shape[0], _p(sp))
    return sp[:g]


def aggregate_groups(sorted_rec: np.ndarray, start_pos: np.ndarray, op: int) -> np.ndarray:
    sorted_rec = np.ascontiguousarray(sorted_rec, np.int32)
    start_pos = np.ascontiguousarray(start_pos, np.int32)
    agg = np.empty(max(start_pos.size, 1), np.int32)
    lib().orc_aggregate_groups(_p(sorted_rec), sorted_rec.shape[0], _p(start_pos), start_pos.size, op, _p(agg))
    return agg[: start_pos.size]


def groupby_cols(key, val, val2=None, lo2=-(2 ** 31), hi2=2 ** 31 - 1, cap=None, mt=False):
    key = np.ascontiguousarray(key, np.int32)
    val = np.ascontiguousarray(val, np.int32)
    v2 = None if val2 is None else np.ascontiguousarray(val2, np.int32)
    cap = key.size if cap is None else cap
    gk = np.empty(max(cap, 1), np.int32)
    gs = np.empty(max(cap, 1), np.int64)
    gc = np.empty(max(cap, 1), np.int64)
    f = lib().orc_groupby_cols_mt if mt else lib().orc_groupby_cols
    g = f(_p(key), _p(val), _p(v2), lo2, hi2, key.size, cap, _p(gk), _p(gs), _p(gc))
    if g < 0:
        raise ValueError("more groups than cap")
    return gk[:g], gs[:g], gc[:g]


def join_filter_sort(rkey, rpay, skey, spay, slo=-(2 ** 31), shi=2 ** 31 - 1, cap=None, mt=False):
    arrs = [np.ascontiguousarray(a, np.int32) for a in (rkey, rpay, skey, spay)]
    rkey, rpay, skey, spay = arrs
    cap = skey.size if cap is None else cap
    ok = np.empty(max(cap, 1), np.int32)
    orp = np.empty(max(cap, 1), np.int32)
    osp = np.empty(max(cap, 1), np.int32)
    f = lib().orc_join_filter_sort_mt if mt else lib().orc_join_filter_sort
    m = f(_p(rkey), _p(rpay), rkey.size, _p(skey), _p(spay), skey.size, slo, shi, cap, _p(ok), _p(orp), _p(osp))
    if m < 0:
        raise ValueError(f"join output {-m - 1} exceeds cap {cap}")
    return ok[:m], orp[:m], osp[:m]


def hash_join_ref(r_pairs: np.ndarray, s_pairs: np.ndarray, cap=None) -> np.ndarray:
    r = np.ascontiguousarray(r_pairs, np.int32)
    s = np.ascontiguousarray(s_pairs, np.int32)
    cap = s.shape[0] * 4 if cap is None else cap
    out = np.empty((max(cap, 1), 2), np.int32)
    m = lib().orc_hash_join_ref(_p(r), r.shape[0], _p(s), s.shape[0], cap, _p(out))
    if m < 0:
        raise ValueError("output exceeds cap")
    return out[:m]


def ref_tool(*args: str) -> str:
    """Run the reference's own generator / validators / planner (compiled
    from the reference sources into oracle/_ref)."""
    res = subprocess.run([str(REF_TOOL), *map(str, args)], capture_output=True, text=True)
    return res.stdout + res.stderr


def mlp_forward(params: np.ndarray, X: np.ndarray) -> np.ndarray:
    p = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(X, np.float32)
    out = np.empty(x.shape[0], np.float64)
    lib().orc_mlp_forward(_p(p), _p(x), x.shape[0], _p(out))
    return out


def mlp_grad(params: np.ndarray, X: np.ndarray, y: np.ndarray):
    """(loss, gradient) of mean((f(X) - y)^2) in double precision."""
    p = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(X, np.float32)
    t = np.ascontiguousarray(y, np.float32)
    g = np.empty(p.size, np.float64)
    loss = lib().orc_mlp_grad(_p(p), _p(x), _p(t), x.shape[0], _p(g))
    return loss, g


def reduce_rec(rec: np.ndarray, op: int) -> int:
    r = np.ascontiguousarray(rec, np.int32)
    return int(lib().orc_reduce_rec(_p(r), r.shape[0], op))


def split_rec(rec: np.ndarray, parts: int):
    r = np.ascontiguousarray(rec, np.int32)
    out = np.empty_like(r)
    bound = np.empty(parts, np.int32)
    lib().orc_split_rec(_p(r), r.shape[0], parts, _p(out), _p(bound))
    return out, bound


# ---- the reference's own OpenCL kernels, run on host cores ------------------
# oracle/_ref/libref_kernels.so (oracle/ref_kernels/, built by build_ref.sh
# only where the reference checkout exists).  They pin the restatement above
# against the reference itself; absent elsewhere (ref_kernels() is None).
REF_KERNELS = HERE / "_ref" / "libref_kernels.so"
_rk = None


def ref_kernels():
    global _rk
    if _rk is None and REF_KERNELS.exists():
        L = ctypes.CDLL(str(REF_KERNELS))
        sig = {
            "ref_filter_rec": [c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p],
            "ref_scan": [c_void_p, c_int, c_void_p],
            "ref_sort_rec": [c_void_p, c_int],
            "ref_groupby_rec": [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p],
            "ref_aggregate": [c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_void_p],
            "ref_hash_join": [c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.restype, f.argtypes = c_int, args
        _rk = L
    return _rk


def _rk_check(st: int, what: str) -> None:
    if st != 0:
        raise ValueError(f"{what}: outside the reference's supported sizes")


def refk_filter_rec(rec: np.ndarray, lo: int, hi: int, num_thread: int = 256, num_block: int = 128) -> np.ndarray:
    """filterImpl (host/host/testFilter.cpp:92-154) over the reference kernels."""
    r = np.ascontiguousarray(rec, np.int32)
    out = np.empty_like(r)
    m = c_int(0)
    _rk_check(ref_kernels().ref_filter_rec(_p(r), r.shape[0], lo, hi, num_thread, num_block, _p(out),
                                           ctypes.byref(m)), "ref_filter_rec")
    return out[: m.value]


def refk_scan(x: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(x, np.int32)
    out = np.empty_like(a)
    _rk_check(ref_kernels().ref_scan(_p(a), a.size, _p(out)), "ref_scan")
    return out


def refk_sort_rec(rec: np.ndarray) -> np.ndarray:
    """radixSortImpl_sm (host/host/testSort.cpp:24-136): bitonic, not stable."""
    r = np.array(rec, np.int32, copy=True, order="C")
    _rk_check(ref_kernels().ref_sort_rec(_p(r), r.shape[0]), "ref_sort_rec")
    return r


def refk_groupby_rec(rec: np.ndarray, num_thread: int = 256, num_block: int = 4):
    """groupByImpl (host/host/testGroupBy.cpp:81-154): (sorted records, startPos)."""
    r = np.ascontiguousarray(rec, np.int32)
    srt = np.empty_like(r)
    sp = np.empty(r.shape[0], np.int32)
    g = c_int(0)
    _rk_check(ref_kernels().ref_groupby_rec(_p(r), r.shape[0], num_thread, num_block, _p(srt), _p(sp),
                                            ctypes.byref(g)), "ref_groupby_rec")
    return srt, sp[: g.value]


def refk_aggregate(sorted_rec: np.ndarray, start_pos: np.ndarray, op: int, num_thread: int = 256) -> np.ndarray:
    """parallelAggregate_kernel chunks (host/host/testAggAfterGB.cpp:127-193)."""
    r = np.ascontiguousarray(sorted_rec, np.int32)
    sp = np.ascontiguousarray(start_pos, np.int32)
    out = np.empty(max(sp.size, 1), np.int32)
    _rk_check(ref_kernels().ref_aggregate(_p(r), r.shape[0], _p(sp), sp.size, op, num_thread, _p(out)),
              "ref_aggregate")
    return out[: sp.size]


def refk_hash_join(r_pairs: np.ndarray, s_pairs: np.ndarray, bucket_num: int = 1024, probe_groups: int = 16):
    """buildHashTable + probeHashTable (kernel/hj_filter_sort/1/hj_filter_sort_op.cl:25-109):
    the (S.value, R.value) pairs in the probe's slot order, holes removed."""
    r = np.ascontiguousarray(r_pairs, np.int32)
    s = np.ascontiguousarray(s_pairs, np.int32)
    fullest = int(np.bincount(r[:, 0].view(np.uint32) & (bucket_num - 1), minlength=bucket_num).max()) if r.size else 1
    out = np.empty((max(s.shape[0], 1), 2), np.int32)
    m = c_int(0)
    _rk_check(ref_kernels().ref_hash_join(_p(r), r.shape[0], _p(s), s.shape[0], bucket_num, max(fullest, 1),
                                          probe_groups, _p(out), ctypes.byref(m)), "ref_hash_join")
    return out[: m.value]
