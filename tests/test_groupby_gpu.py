"""GPU parity: group-by (sorted contract + per-group aggregates, bit-exact) and
the column hash group-by with int64 SUM + COUNT, plain and fused with the
value2 predicate (bit-exact; compared in key order)."""
import numpy as np
import pytest
import torch

from query_on_opencl_fpga_gb300 import datagen
from query_on_opencl_fpga_gb300.api import QG_ORDER_KEY, QG_ORDER_NONE

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_groupby_rec_golden(ctx, orc, golden):
    meta, arrs = golden
    c = meta["cases"]["groupby"]
    rin = orc.generate_rand(64, c["n"], 0)
    rin[:, 1] = np.mod(rin[:, 1], 64)
    srt, sp = ctx.groupby_rec(dev(rin))
    assert np.array_equal(sp.cpu().numpy(), arrs["groupby_startpos"])
    assert np.array_equal(srt.cpu().numpy()[:, 1], orc.sort_rec(rin)[:, 1])


@pytest.mark.parametrize("op,name", [(0, "sum"), (1, "max"), (2, "min"), (3, "avg")])
def test_aggregate_golden(ctx, orc, golden, op, name):
    meta, arrs = golden
    c = meta["cases"]["aggregate"]
    rin = orc.generate_rand(50, c["n"], 0)
    rin[:, 1] = np.mod(rin[:, 1], 50)
    srt, sp = ctx.groupby_rec(dev(rin))
    agg = ctx.aggregate_groups(srt, sp, op).cpu().numpy()
    assert np.array_equal(agg, arrs[f"agg_{name}"])


@pytest.mark.parametrize("n,groups", [(1, 1), (5, 2), (4097, 7), (100003, 1000), (1 << 20, 40000),
                                      (300000, 1)])
@pytest.mark.parametrize("op", [0, 1, 2, 3])
def test_aggregate_sizes(ctx, orc, n, groups, op):
    rng = np.random.default_rng(n + op)
    rin = np.stack([rng.integers(-(2 ** 31), 2 ** 31, n, dtype=np.int64),
                    rng.integers(0, groups, n)], 1).astype(np.int32)
    srt, sp = ctx.groupby_rec(dev(rin))
    srt_h = srt.cpu().numpy()
    sp_h = sp.cpu().numpy()
    exp_sorted = orc.sort_rec(rin)
    assert np.array_equal(srt_h[:, 1], exp_sorted[:, 1])
    assert np.array_equal(sp_h, orc.group_startpos(exp_sorted))
    agg = ctx.aggregate_groups(srt, sp, op).cpu().numpy()
    assert np.array_equal(agg, orc.aggregate_groups(srt_h, sp_h, op))


def check_groups(got, exp):
    gk, gs, gc = [t.cpu().numpy() for t in got]
    ek, es, ec = exp
    assert np.array_equal(gk, ek)
    assert np.array_equal(gs, es)
    assert np.array_equal(gc, ec)


@pytest.mark.parametrize("n,groups,fused", [(1, 1, False), (100, 7, True), (4099, 4099, False),
                                            (1 << 18, 1 << 12, True), (1 << 20, 1 << 17, False),
                                            (1 << 20, 1 << 17, True)])
def test_groupby_cols_small(ctx, orc, n, groups, fused):
    d = datagen.config1_groupby(n, groups, seed=n)
    key, val, val2 = d["key"].numpy(), d["val"].numpy(), d["val2"].numpy()
    v2 = val2 if fused else None
    got = ctx.groupby_cols(dev(key), dev(val), dev(v2) if fused else None, d["lo2"], d["hi2"],
                           cap=max(groups, 1) * 2)
    exp = orc.groupby_cols(key, val, v2, d["lo2"], d["hi2"])
    check_groups(got, exp)


def test_groupby_cols_extreme_values(ctx, orc):
    # key -1 (all-ones) and INT_MIN/INT_MAX values exercise the shared-memory
    # sentinel path and the int64 sum.
    rng = np.random.default_rng(4)
    n = 1 << 16
    key = rng.choice(np.array([-1, 0, 1, 2 ** 31 - 1, -(2 ** 31), 12345], np.int32), n)
    val = rng.choice(np.array([-(2 ** 31), 2 ** 31 - 1, 0, -1], np.int32), n)
    got = ctx.groupby_cols(dev(key), dev(val), cap=16)
    check_groups(got, orc.groupby_cols(key, val))


def test_groupby_cols_unordered_is_permutation(ctx, orc):
    d = datagen.config1_groupby(1 << 20, 1 << 15, seed=3)
    key, val = d["key"].numpy(), d["val"].numpy()
    gk, gs, gc = ctx.groupby_cols(dev(key), dev(val), cap=1 << 16, order=QG_ORDER_NONE)
    order = np.argsort(gk.cpu().numpy().view(np.uint32))
    got = (gk.cpu()[order], gs.cpu()[order], gc.cpu()[order])
    check_groups(got, orc.groupby_cols(key, val))


def test_groupby_cols_capacity(ctx):
    from query_on_opencl_fpga_gb300 import QGError

    key = torch.arange(5000, dtype=torch.int32, device="cuda")
    with pytest.raises(QGError) as e:
        ctx.groupby_cols(key, key, cap=100)
    assert e.value.status in (3, 4)
    # usable afterwards (the table is cleared after an error)
    gk, gs, gc = ctx.groupby_cols(key[:50], key[:50], cap=100)
    assert gk.numel() == 50 and int(gc.sum()) == 50


@pytest.mark.parametrize("fused", [False, True])
def test_groupby_config1_full_size(ctx, orc, fused):
    # Full config-1 size: 64M rows, Zipf(1.0) over 1M groups, bit-exact.
    d = datagen.config1_groupby(1 << 26, 1 << 20, seed=0, device="cuda")
    got = ctx.groupby_cols(d["key"], d["val"], d["val2"] if fused else None, d["lo2"], d["hi2"],
                           cap=1 << 21)
    key, val, val2 = d["key"].cpu().numpy(), d["val"].cpu().numpy(), d["val2"].cpu().numpy()
    exp = orc.groupby_cols(key, val, val2 if fused else None, d["lo2"], d["hi2"], cap=1 << 21, mt=True)
    check_groups(got, exp)
    # checksum of checksums: total count and sum equal the filtered column sums
    m = (val2 <= 499) if fused else np.ones(key.size, bool)
    assert int(got[2].sum()) == int(m.sum())
    assert int(got[1].sum()) == int(val[m].astype(np.int64).sum())


@pytest.fixture
def knobs(ctx):
    yield lambda *a: ctx.check(ctx.lib.qg_groupby_set_knobs(*a), "knobs")
    ctx.lib.qg_groupby_set_knobs(0, 13, 0, 0)


@pytest.mark.parametrize("fused", [False, True])
def test_groupby_global_table_path(ctx, orc, knobs, fused):
    # mode 1: the single-pass global-table kernel alone
    knobs(1, 13, 0, 0)
    d = datagen.config1_groupby(1 << 20, 1 << 16, seed=11)
    key, val, val2 = d["key"].numpy(), d["val"].numpy(), d["val2"].numpy()
    v2 = val2 if fused else None
    got = ctx.groupby_cols(dev(key), dev(val), dev(v2) if fused else None, d["lo2"], d["hi2"], cap=1 << 17)
    check_groups(got, orc.groupby_cols(key, val, v2, d["lo2"], d["hi2"]))


def test_groupby_spill_overflow_falls_back(ctx, orc, knobs):
    # two-pass path (mode 3), bucket capacity 1 overflows at once: the call is
    # redone on the global table
    knobs(3, 8, 4, 1)
    d = datagen.config1_groupby(1 << 18, 1 << 14, seed=12)
    key, val = d["key"].numpy(), d["val"].numpy()
    got = ctx.groupby_cols(dev(key), dev(val), cap=1 << 15)
    check_groups(got, orc.groupby_cols(key, val))


def test_groupby_async_overflow_reports_table_full(ctx, knobs):
    from ctypes import c_void_p

    from query_on_opencl_fpga_gb300 import QGError

    knobs(3, 8, 4, 1)
    n = 1 << 16
    key = torch.arange(n, dtype=torch.int32, device="cuda")
    out_k = torch.empty(n, dtype=torch.int32, device="cuda")
    out_s = torch.empty(n, dtype=torch.int64, device="cuda")
    out_c = torch.empty(n, dtype=torch.int64, device="cuda")
    d_num = torch.zeros(1, dtype=torch.int64, device="cuda")
    p = lambda t: c_void_p(t.data_ptr())  # noqa: E731
    st = ctx.lib.qg_groupby_cols_async(ctx.handle, p(key), p(key), c_void_p(0), 0, 0, n, p(out_k), p(out_s),
                                       p(out_c), n, QG_ORDER_NONE, p(d_num))
    assert st == 0
    with pytest.raises(QGError) as e:
        ctx.device_check()
    assert e.value.status == 4


@pytest.mark.parametrize("n,groups,fused", [(1, 1, False), (5000, 37, True), (1 << 19, 1 << 16, False)])
def test_groupby_async_key_order(ctx, orc, n, groups, fused):
    # The sync-free form sorts by key on the device (digit counts from the merge,
    # group count read by the kernels); the count comes back in d_num.
    from ctypes import c_void_p

    d = datagen.config1_groupby(n, groups, seed=n + 3)
    key, val, val2 = d["key"].numpy(), d["val"].numpy(), d["val2"].numpy()
    cap = 2 * groups
    k, v, w = dev(key), dev(val), dev(val2)
    out = [torch.empty(cap, dtype=t, device="cuda") for t in (torch.int32, torch.int64, torch.int64)]
    d_num = torch.zeros(1, dtype=torch.int64, device="cuda")
    p = lambda t: c_void_p(t.data_ptr())  # noqa: E731
    st = ctx.lib.qg_groupby_cols_async(ctx.handle, p(k), p(v), p(w) if fused else c_void_p(0), d["lo2"], d["hi2"],
                                       n, p(out[0]), p(out[1]), p(out[2]), cap, QG_ORDER_KEY, p(d_num))
    assert st == 0
    ctx.device_check()
    g = int(d_num.item())
    check_groups([t[:g] for t in out], orc.groupby_cols(key, val, val2 if fused else None, d["lo2"], d["hi2"]))


@pytest.mark.parametrize("mode", [0, 2, 3])
@pytest.mark.parametrize("hot,parts", [(8, 1), (10, 6), (13, 12), (13, 13)])
def test_groupby_knob_sweep(ctx, orc, knobs, hot, parts, mode):
    knobs(mode, hot, parts, 0)
    d = datagen.config1_groupby(1 << 19, 1 << 15, seed=hot + parts)
    key, val, val2 = d["key"].numpy(), d["val"].numpy(), d["val2"].numpy()
    got = ctx.groupby_cols(dev(key), dev(val), dev(val2), d["lo2"], d["hi2"], cap=1 << 16)
    check_groups(got, orc.groupby_cols(key, val, val2, d["lo2"], d["hi2"]))


@pytest.mark.parametrize("cap", [1 << 20, 1 << 21])
def test_groupby_config1_paths(ctx, knobs, cap):
    # The full config-1 input (64M rows, Zipf(1.0) over 2^20 keys) stays on the
    # dense-window path by default (every key inside the sampled window), and
    # on the two-pass path without a fallback when that path is chosen (mode 3)
    # with the output capacity the bench passes (the key domain, 1024 spill
    # partitions) and with twice that (2048 partitions).
    d = datagen.config1_groupby(1 << 26, 1 << 20, seed=0, device="cuda")
    for v2 in (None, d["val2"]):
        ctx.groupby_cols(d["key"], d["val"], v2, d["lo2"], d["hi2"], cap=cap, order=QG_ORDER_NONE)
        st = ctx.groupby_stats()
        assert st["path"] == "dense" and st["bucket_cap"] == 0, st
    knobs(3, 13, 0, 0)
    for v2 in (None, d["val2"]):
        ctx.groupby_cols(d["key"], d["val"], v2, d["lo2"], d["hi2"], cap=cap, order=QG_ORDER_NONE)
        st = ctx.groupby_stats()
        assert st["path"] == "two_pass" and st["flags"] == 0, st
        assert st["fullest_bucket"] <= st["bucket_cap"], st


def test_groupby_config1_headline_calls_repeated(ctx, orc):
    # The bench's step exactly: group-by then fused filter_aggregation over the
    # same 64M-row config-1 columns, cap = 2^20 (the key domain), key order,
    # caller-owned output columns, three steps in a row on one context; every
    # call bit-exact against the oracle.
    d = datagen.config1_groupby(1 << 26, 1 << 20, seed=0, device="cuda")
    key, val, val2 = d["key"].cpu().numpy(), d["val"].cpu().numpy(), d["val2"].cpu().numpy()
    cap = 1 << 20
    exp = [orc.groupby_cols(key, val, None, d["lo2"], d["hi2"], cap=1 << 21, mt=True),
           orc.groupby_cols(key, val, val2, d["lo2"], d["hi2"], cap=1 << 21, mt=True)]
    outs = [tuple(torch.empty(cap, dtype=t, device="cuda") for t in (torch.int32, torch.int64, torch.int64))
            for _ in range(2)]
    for _ in range(3):
        for i, v2 in enumerate((None, d["val2"])):
            got = ctx.groupby_cols(d["key"], d["val"], v2, d["lo2"], d["hi2"], cap=cap, order=QG_ORDER_KEY,
                                   out=outs[i])
            check_groups(got, exp[i])
            assert ctx.groupby_stats()["path"] == "dense"
    ctx.release_out_buffers()


def _dense_case(ctx, orc, key, val, val2=None, lo2=0, hi2=0, cap=None, path=None, order=QG_ORDER_KEY):
    cap = cap or max(1, key.size)
    got = ctx.groupby_cols(dev(key), dev(val), dev(val2) if val2 is not None else None, lo2, hi2, cap=cap,
                           order=order)
    exp = orc.groupby_cols(key, val, val2, lo2, hi2)
    if order == QG_ORDER_NONE:
        o = np.argsort(got[0].cpu().numpy().view(np.uint32), kind="stable")
        got = tuple(t.cpu()[o] for t in got)
    check_groups(got, exp)
    if path is not None:
        assert ctx.groupby_stats()["path"] == path, ctx.groupby_stats()


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7, 4095, 4097, 65537, (1 << 18) + 3, (1 << 18) + 1027])
def test_groupby_dense_ragged_sizes(ctx, orc, n):
    # every row sampled (n <= 2^18) or runs spread over the column; tails of
    # 1-3 rows after the 4-row vectors
    rng = np.random.default_rng(n)
    key = (rng.zipf(1.3, n) % 50000).astype(np.int32) + 1000
    val = rng.integers(0, 1000, n).astype(np.int32)
    _dense_case(ctx, orc, key, val, path="dense")
    val2 = rng.integers(0, 1000, n).astype(np.int32)
    _dense_case(ctx, orc, key, val, val2, -(2 ** 31), 499, path="dense")


def test_groupby_dense_wide_and_signed_values(ctx, orc):
    # values outside [0, fast_max] (negative, INT_MIN/INT_MAX) take the int64
    # side table, mixed with small ones on the same keys; heavy and light keys
    rng = np.random.default_rng(5)
    n = 1 << 20
    key = np.where(rng.random(n) < 0.5, rng.integers(0, 64, n), rng.integers(0, 1 << 20, n)).astype(np.int32)
    val = rng.choice(np.array([-(2 ** 31), 2 ** 31 - 1, -1, 0, 5, 2047, 2048, 1 << 30], np.int64), n)
    val = np.where(rng.random(n) < 0.5, val, rng.integers(0, 1000, n)).astype(np.int32)
    _dense_case(ctx, orc, key, val, path="dense")
    _dense_case(ctx, orc, key, val, val, -(2 ** 31), 100, path="dense")
    # the next call on the same context starts from a clean table
    _dense_case(ctx, orc, key[: n // 3], rng.integers(0, 1000, n // 3).astype(np.int32), path="dense")


@pytest.mark.parametrize("single", [1, 0])
@pytest.mark.parametrize("n", [5, 4097, (1 << 18) + 3, (1 << 22) + 1])
def test_groupby_dense_single_and_four_launches(ctx, orc, n, single):
    # The dense-window steps as one cooperative launch (grid barriers) and as
    # four launches give the same exact groups, plain and fused, on sizes
    # below and above the every-row sample; repeated calls on one context
    # start from a clean table either way.
    ctx.groupby_set_single_launch(bool(single))
    try:
        rng = np.random.default_rng(n + single)
        key = (rng.zipf(1.2, n) % 200000).astype(np.int32) - 300000  # negative: high unsigned keys
        val = np.where(rng.random(n) < 0.01, rng.integers(-(2 ** 31), 2 ** 31 - 1, n),
                       rng.integers(0, 1000, n)).astype(np.int32)
        val2 = rng.integers(0, 1000, n).astype(np.int32)
        for _ in range(2):
            _dense_case(ctx, orc, key, val, path="dense")
            _dense_case(ctx, orc, key, val, val2, -(2 ** 31), 499, path="dense")
    finally:
        ctx.groupby_set_single_launch(False)


@pytest.mark.parametrize("single", [0, 1])
def test_groupby_dense_timeout_reports_and_recovers(ctx, orc, single):
    # Poll limit 0: the emit's look-back over its chunks (four launches) gives
    # up at once and the call reports a timeout; the single launch's grid
    # barriers give up unless every CTA has already arrived.  Either way no
    # hang and no fault, and the next call with the default limit is exact
    # (the error path re-zeroes the table arena and the state words).
    from query_on_opencl_fpga_gb300 import QGError

    rng = np.random.default_rng(77)
    n = 1 << 22
    key = (rng.zipf(1.2, n) % 100000).astype(np.int32)
    val = rng.integers(0, 1000, n).astype(np.int32)
    exp = orc.groupby_cols(key, val, None, 0, 0)
    ctx.groupby_set_single_launch(bool(single))
    try:
        ctx.set_spin_limit(0)
        try:
            if single:
                try:
                    check_groups(ctx.groupby_cols(dev(key), dev(val), None, 0, 0, cap=n), exp)
                except QGError as e:
                    assert e.status == 5
            else:
                with pytest.raises(QGError) as e:
                    ctx.groupby_cols(dev(key), dev(val), None, 0, 0, cap=n)
                assert e.value.status == 5
        finally:
            ctx.set_spin_limit(1 << 22)
        for _ in range(2):
            _dense_case(ctx, orc, key, val, path="dense")
    finally:
        ctx.groupby_set_single_launch(False)


@pytest.mark.parametrize("n,nkeys,vmax", [(1 << 22, 8, 600_000), (1 << 20, 4, 1 << 23), (1 << 22, 1, None)])
def test_groupby_dense_heavy_slot_bounds(ctx, orc, n, nkeys, vmax):
    # A few keys take every row, so each CTA's heavy-key slots take thousands
    # of adds per key, with values up to and past the bound on values the
    # packed count/sum words take (the largest such value on every row, for
    # one key), and at 2^20 rows values of 2^21 and more.
    rng = np.random.default_rng(n + nkeys)
    key = (rng.integers(0, nkeys, n) * 7919 + 12345).astype(np.int32)
    if vmax is None:  # the largest fast value for n rows on every row
        shift = 64 - n.bit_length()
        val = np.full(n, ((1 << shift) - 1) // n, np.int64)
        val = np.minimum(val, 2 ** 31 - 1).astype(np.int32)
    else:
        val = rng.integers(0, vmax, n).astype(np.int32)
    _dense_case(ctx, orc, key, val, path="dense")
    _dense_case(ctx, orc, key, val, val, -(2 ** 31), vmax // 2 if vmax else 2 ** 31 - 1, path="dense")


@pytest.mark.parametrize("lo", [0, 2 ** 31 - 1000, 2 ** 32 - 3000])
def test_groupby_dense_window_positions(ctx, orc, lo):
    # keys from 0 up, across the signed boundary, and at the top of the
    # unsigned range (the window is clamped to end at 2^32); key order is
    # ascending unsigned
    rng = np.random.default_rng(lo & 0xffff)
    n = 1 << 19
    key = (lo + rng.integers(0, 3000, n)).astype(np.uint32).view(np.int32)
    val = rng.integers(-5, 1000, n).astype(np.int32)
    _dense_case(ctx, orc, key, val, path="dense")


def test_groupby_dense_outside_window_falls_back(ctx, orc):
    # Two rows far from the sampled key range, placed where no sample run
    # reads them: the dense pass counts them as outside and the call is
    # answered by the two-pass path, exactly.  Keys spread over more than
    # 2^21 values get no window at all.
    rng = np.random.default_rng(6)
    n = 1 << 22
    key = rng.integers(100, 100 + 50000, n).astype(np.int32)
    runs = 1024
    starts = np.array([(n - 256) * r // (runs - 1) for r in range(runs)])
    gap = 300  # after run 0 ([0, 256)), before run 1
    assert not np.any((starts <= gap + 1) & (gap < starts + 256))
    key[gap], key[gap + 1] = 2 ** 30, -5
    val = rng.integers(0, 1000, n).astype(np.int32)
    _dense_case(ctx, orc, key, val, path="two_pass")
    wide = rng.integers(-(2 ** 31), 2 ** 31, 1 << 18).astype(np.int32)
    _dense_case(ctx, orc, wide, rng.integers(0, 1000, wide.size).astype(np.int32), path="two_pass")
    # and the dense path applies again on the next call
    _dense_case(ctx, orc, key[:gap], val[:gap], path="dense")


def test_groupby_dense_capacity_and_unordered(ctx, orc):
    from query_on_opencl_fpga_gb300 import QGError

    rng = np.random.default_rng(8)
    n = 1 << 18
    key = rng.integers(0, 3000, n).astype(np.int32)
    val = rng.integers(0, 1000, n).astype(np.int32)
    g = np.unique(key).size
    with pytest.raises(QGError) as e:
        ctx.groupby_cols(dev(key), dev(val), cap=g - 1)
    assert e.value.status == 3
    _dense_case(ctx, orc, key, val, cap=g, path="dense")
    _dense_case(ctx, orc, key, val, cap=g, path="dense", order=QG_ORDER_NONE)


def test_groupby_cols_into_caller_buffers(ctx, orc):
    # out=: the caller's (key, sum, count) buffers, reused across calls
    d = datagen.config1_groupby(1 << 18, 1 << 12, seed=21)
    key, val, val2 = d["key"].numpy(), d["val"].numpy(), d["val2"].numpy()
    cap = 1 << 13
    out = (torch.empty(cap, dtype=torch.int32, device="cuda"), torch.empty(cap, dtype=torch.int64, device="cuda"),
           torch.empty(cap, dtype=torch.int64, device="cuda"))
    for v2 in (None, val2):
        got = ctx.groupby_cols(dev(key), dev(val), dev(v2) if v2 is not None else None, d["lo2"], d["hi2"], cap=cap,
                               out=out)
        assert got[0].data_ptr() == out[0].data_ptr()
        check_groups(got, orc.groupby_cols(key, val, v2, d["lo2"], d["hi2"]))
    with pytest.raises(ValueError):
        ctx.groupby_cols(dev(key), dev(val), cap=cap, out=(out[0][:10], out[1], out[2]))
    # after the remembered sets are dropped the same buffers validate again
    ctx.release_out_buffers()
    got = ctx.groupby_cols(dev(key), dev(val), cap=cap, out=out)
    check_groups(got, orc.groupby_cols(key, val))


def _key_order_keys(rng, n, kind):
    if kind == "dense":  # unsigned-contiguous across the signed boundary
        return rng.integers(2 ** 31 - 3000, 2 ** 31 + 3000, n).astype(np.uint32).view(np.int32)
    if kind == "low":  # from key 0 up
        k = rng.integers(0, 5000, n)
        k[0] = 0
        return k.astype(np.int32)
    if kind == "wide":  # -5..5: the unsigned range is nearly 2^32
        return rng.integers(-5, 6, n).astype(np.int32)
    k = rng.integers(7, 7 + (1 << 27) - 1, n)
    k[0], k[1] = 7, 7 + (1 << 27) - 1 + (kind == "over")  # 2^27 values ("edge"), or one more
    return k.astype(np.int32)


def _check_key_order_sequence(c, orc, kinds, seed):
    rng = np.random.default_rng(seed)
    n = 1 << 17
    for kind in kinds:
        key = _key_order_keys(rng, n, kind)
        val = rng.integers(-1000, 1000, n).astype(np.int32)
        got = c.groupby_cols(dev(key), dev(val), cap=n)
        check_groups(got, orc.groupby_cols(key, val))
        fused = c.groupby_cols(dev(key), dev(val), dev(val), -10, 500, cap=n)
        check_groups(fused, orc.groupby_cols(key, val, val, -10, 500))


def test_groupby_key_order_dense_and_wide_ranges(ctx, orc):
    # Key order places the groups by rank in a bitmap over a window of 2^27
    # keys, which the merge fills; the window follows the context's previous
    # key-ordered call.  Keys outside it (placed by a sort after the count),
    # or spread wider than 2^27 (sorted on the device from then on), take the
    # other paths.  The sequence takes every transition, both sides of the
    # 2^27 limit and a window whose last word holds the largest key.
    kinds = ["dense", "dense", "wide", "wide", "dense", "dense", "low", "low", "edge", "edge", "over",
             "over", "edge", "edge", "dense", "dense"]
    _check_key_order_sequence(ctx, orc, kinds, 9)


def test_groupby_key_order_fresh_context_window(orc):
    # A fresh context's first window starts at key 0: keys far from it fall
    # back (and the merge's bits in the window are cleared), after which the
    # window follows the keys and every later call is exact.
    from query_on_opencl_fpga_gb300.api import Context

    c = Context()
    try:
        _check_key_order_sequence(c, orc, ["dense", "dense", "low", "dense", "edge", "low", "low"], 10)
    finally:
        c.close()
